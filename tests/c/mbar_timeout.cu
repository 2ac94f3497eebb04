// mbar_timeout.cu -- the bounded wait of the bulk-copy staging, made to run out.
//
// The two-sided chain kernels wait for their bulk copies on mbarriers with
// mbar_wait (spike_common.cuh), which gives up after a fixed number of polls
// instead of spinning forever.  This kernel waits on a barrier that nothing
// ever arrives on (no copy is issued, no thread arrives), so the wait must
// return false; the kernel then records the outcome and returns normally,
// leaving the context usable.  Built by tests/test_gpu_mbar_timeout.py with
// nvcc for sm_103a; test code only.
#include "spike_common.cuh"

__global__ void k_wait_never(int *out)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    const bool landed = mbar_wait(&bar, 0); // phase 0 never completes
    if (__syncthreads_or(!landed) && threadIdx.x == 0) out[0] = 1;
    if (threadIdx.x == 0) out[1] = landed ? 1 : 0;
}

// the same barrier with the expected bytes delivered: the wait succeeds
__global__ void k_wait_copy(const float *src, float *dst, int *out)
{
    __shared__ __align__(128) float buf[256];
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, sizeof buf);
        bulk_g2s(buf, src, sizeof buf, &bar);
    }
    const bool landed = mbar_wait(&bar, 0);
    if (landed) dst[threadIdx.x] = buf[threadIdx.x];
    if (threadIdx.x == 0) out[2] = landed ? 1 : 0;
}

// returns 0 or the CUDA error code; flags: [timed out, landed (never), landed (copy)]
extern "C" int mbar_check(int *flags, float *ms)
{
    int *d = nullptr;
    float *src = nullptr, *dst = nullptr;
    cudaError_t e = cudaMalloc(&d, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&src, 256 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dst, 256 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(d, 0, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(src, 0, 256 * sizeof(float));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    if (e == cudaSuccess) {
        cudaEventRecord(a);
        k_wait_never<<<1, 64>>>(d);
        cudaEventRecord(b);
        k_wait_copy<<<1, 256>>>(src, dst, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(flags, d, 3 * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    cudaFree(src);
    cudaFree(dst);
    return (int)e;
}
