// rcp_check.cu -- device check of the factor-precision reciprocal.
//
// sc_rcp_fast (spike_common.cuh) forms 1/a for the FP32 tile inverses as the
// hardware approximation `rcp.approx.ftz.f32` followed by one Newton-Raphson
// step r' = r + r (1 - a r) (the textbook iteration for 1/a).  This kernel
// evaluates it beside the correctly rounded reciprocal __frcp_rn on the same
// inputs, so that the test can bound their distance in units in the last place.
// Built by tests/test_gpu_rcp.py with nvcc for sm_103a; test code only.
#include "spike_common.cuh"

__global__ void k_rcp_check(const float *in, float *fast, float *rn, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        fast[i] = sc_rcp_fast(in[i]);
        rn[i] = __frcp_rn(in[i]);
    }
}

// host arrays in, host arrays out; returns 0 or the CUDA error code
extern "C" int rcp_check(const float *h_in, float *h_fast, float *h_rn, int n)
{
    float *d = nullptr;
    const size_t bytes = sizeof(float) * (size_t)n;
    cudaError_t e = cudaMalloc(&d, 3 * bytes);
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpy(d, h_in, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_rcp_check<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h_fast, d + n, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_rn, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return (int)e;
}
