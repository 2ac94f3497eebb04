// spike_util.cu -- device plumbing, CSR analysis and the FP64 residual.
//
//   k_analyze    bandwidth (matrix_ComputeBandwidth, OpenMP/spike_algebra.c
//                :56-95) plus CSR validation in one pass over colind: rowptr
//                monotone and inside [0, nnz], columns inside [0, n) and
//                strictly increasing within a row.  Rows whose rowptr entries
//                are out of range are flagged and never dereferenced.
//   k_residual   r = b - A x and ||r||^2 per column in FP64 / complex128
//                (ComputeResidualOfLinearSystem, OpenMP/spike_algebra.c:97-151,
//                which uses MKL csrgemv for the first five columns only).
#include "spike_common.cuh"

#include <stdio.h>
#include <stdlib.h>

static thread_local cudaError_t g_last_cuda = cudaSuccess;

static int ck(cudaError_t e)
{
    if (e != cudaSuccess) {
        g_last_cuda = e;
        return SPK_ECUDA;
    }
    return SPK_OK;
}

extern "C" const char *spk_cuda_error_string(void) { return cudaGetErrorString(g_last_cuda); }

extern "C" int spk_device_count(void)
{
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}
extern "C" int spk_current_device(void)
{
    int d = -1;
    if (cudaGetDevice(&d) != cudaSuccess) return -1;
    return d;
}
extern "C" int spk_sm_count(void)
{
    int d = spk_current_device(), v = 0;
    if (d < 0 || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess) return 0;
    return v;
}
extern "C" int spk_malloc(void **p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 256;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        g_last_cuda = e;
        cudaGetLastError();
        *p = nullptr;
        return SPK_EMEM;
    }
    return SPK_OK;
}
extern "C" void spk_free(void *p)
{
    if (p) cudaFree(p);
}
extern "C" int spk_host_register(void *p, size_t bytes)
{
    cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SPK_ECUDA;
    }
    return SPK_OK;
}
extern "C" int spk_host_unregister(void *p)
{
    cudaError_t e = cudaHostUnregister(p);
    if (e != cudaSuccess) cudaGetLastError();
    return e == cudaSuccess ? SPK_OK : SPK_ECUDA;
}
extern "C" int spk_stream_create(void **stream)
{
    cudaStream_t s;
    int r = ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = r == SPK_OK ? (void *)s : nullptr;
    return r;
}
extern "C" void spk_stream_destroy(void *stream)
{
    if (stream) cudaStreamDestroy((cudaStream_t)stream);
}
extern "C" int spk_stream_sync(void *stream) { return ck(cudaStreamSynchronize((cudaStream_t)stream)); }
extern "C" int spk_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream)
{
    return ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
}
extern "C" int spk_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream)
{
    return ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
}
extern "C" int spk_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream)
{
    return ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
}
extern "C" int spk_memset(void *dst, int v, size_t bytes, void *stream)
{
    return ck(cudaMemsetAsync(dst, v, bytes, (cudaStream_t)stream));
}

// ------------------------------------------------------------ analysis
__global__ void k_analyze(int n, long long nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
                          int *out)
{
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    int ku = 0, kl = 0;
    unsigned flags = 0;
    for (long long r = warp; r < n; r += nwarps) {
        const long long t0 = rowptr[r], t1 = rowptr[r + 1];
        if (t0 < 0 || t1 > nnz || t1 < t0) {
            flags |= SPK_DEV_ERR_CSR;
            continue;
        }
        for (long long t = t0 + lane; t < t1; t += 32) {
            const int c = colind[t];
            if (c < 0 || c >= n) {
                flags |= SPK_DEV_ERR_CSR;
                continue;
            }
            if (t > t0 && colind[t - 1] >= c) flags |= SPK_DEV_ERR_CSR;
            ku = max(ku, c - (int)r);
            kl = max(kl, (int)r - c);
        }
    }
    if (warp == 0 && lane == 0 && (rowptr[0] != 0 || rowptr[n] != nnz)) flags |= SPK_DEV_ERR_CSR;
    for (int o = 16; o > 0; o >>= 1) {
        ku = max(ku, __shfl_xor_sync(0xffffffffu, ku, o));
        kl = max(kl, __shfl_xor_sync(0xffffffffu, kl, o));
        flags |= __shfl_xor_sync(0xffffffffu, flags, o);
    }
    if (lane == 0) {
        atomicMax(&out[0], ku);
        atomicMax(&out[1], kl);
        if (flags) atomicOr((unsigned *)&out[2], flags);
    }
}

extern "C" int spk_analyze(int n, long long nnz, const int *d_rowptr, const int *d_colind, int *d_out, int *out,
                           void *stream, long long *launches)
{
    cudaStream_t st = (cudaStream_t)stream;
    int r = ck(cudaMemsetAsync(d_out, 0, 4 * sizeof(int), st));
    if (r == SPK_OK && n > 0) {
        const long long warps_needed = n;
        long long blocks = (warps_needed * 32 + 255) / 256;
        if (blocks > 152 * 16) blocks = 152 * 16;
        k_analyze<<<(unsigned)blocks, 256, 0, st>>>(n, nnz, d_rowptr, d_colind, d_out);
        r = ck(cudaGetLastError());
        if (launches) (*launches)++;
    }
    if (r == SPK_OK) r = ck(cudaMemcpyAsync(out, d_out, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
    if (r == SPK_OK) r = ck(cudaStreamSynchronize(st));
    return r;
}

// ------------------------------------------------------------ conversions
__global__ void k_widen(const float *__restrict__ s, double *d, long long count)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < count; q += (long long)gridDim.x * blockDim.x)
        d[q] = (double)s[q];
}
__global__ void k_narrow(const double *__restrict__ s, float *d, long long count)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < count; q += (long long)gridDim.x * blockDim.x)
        d[q] = (float)s[q];
}
extern "C" int spk_widen(const void *src, void *dst, long long count, int is_complex, void *stream, long long *launches)
{
    const long long c = count * (is_complex ? 2 : 1);
    if (c == 0) return SPK_OK;
    k_widen<<<1024, 256, 0, (cudaStream_t)stream>>>((const float *)src, (double *)dst, c);
    if (launches) (*launches)++;
    return ck(cudaGetLastError());
}
extern "C" int spk_narrow(const void *src, void *dst, long long count, int is_complex, void *stream, long long *launches)
{
    const long long c = count * (is_complex ? 2 : 1);
    if (c == 0) return SPK_OK;
    k_narrow<<<1024, 256, 0, (cudaStream_t)stream>>>((const double *)src, (float *)dst, c);
    if (launches) (*launches)++;
    return ck(cudaGetLastError());
}

// ------------------------------------------------------------ residual
// G lanes per row; per-column squared norms reduced in shared memory and
// added to norms[] once per CTA.
constexpr int RES_MAXH = 32;

template <class H, int G>
__global__ void __launch_bounds__(256)
    k_residual(int n, const int *__restrict__ rowptr, const int *__restrict__ colind, const H *__restrict__ aij,
               const H *__restrict__ x, const H *__restrict__ b, H *r, int h0, int nr, int want_b, double *norms,
               int nrhs_total)
{
    __shared__ double sr[RES_MAXH], sb[RES_MAXH];
    for (int q = threadIdx.x; q < RES_MAXH; q += blockDim.x) sr[q] = sb[q] = 0.0;
    __syncthreads();
    const int sub = threadIdx.x % G;
    // rows are walked warp-uniformly (every lane runs every iteration) so the
    // shuffles below always see the full warp
    constexpr int RPW = 32 / G; // rows per warp per iteration
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    double lr[RES_MAXH], lb[RES_MAXH];
    for (int h = 0; h < nr; h++) lr[h] = lb[h] = 0.0;
    for (long long base = warp * RPW; base < n; base += nwarps * RPW) {
        const long long row = base + lane / G;
        const bool valid = row < n;
        const int t0 = valid ? rowptr[row] : 0, t1 = valid ? rowptr[row + 1] : 0;
        for (int h = 0; h < nr; h++) {
            const H *xh = x + (size_t)(h0 + h) * n;
            H acc = sc_zero<H>();
            for (int t = t0 + sub; t < t1; t += G) acc = madd(acc, aij[t], xh[colind[t]]);
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) {
                if constexpr (sizeof(H) == 8) {
                    acc = acc + __shfl_xor_sync(0xffffffffu, acc, o);
                } else {
                    H other;
                    const unsigned *srcw = (const unsigned *)&acc;
                    unsigned *dstw = (unsigned *)&other;
#pragma unroll
                    for (int w = 0; w < (int)(sizeof(H) / 4); w++) dstw[w] = __shfl_xor_sync(0xffffffffu, srcw[w], o);
                    acc = acc + other;
                }
            }
            if (sub == 0 && valid) {
                const H bv = b[(size_t)(h0 + h) * n + row];
                const H rv = bv - acc;
                r[(size_t)(h0 + h) * n + row] = rv;
                lr[h] += sc_abs2(rv);
                if (want_b) lb[h] += sc_abs2(bv);
            }
        }
    }
    if (sub == 0)
        for (int h = 0; h < nr; h++) {
            atomicAdd(&sr[h], lr[h]);
            if (want_b) atomicAdd(&sb[h], lb[h]);
        }
    __syncthreads();
    for (int h = threadIdx.x; h < nr; h += blockDim.x) {
        atomicAdd(&norms[h0 + h], sr[h]);
        if (want_b) atomicAdd(&norms[nrhs_total + h0 + h], sb[h]);
    }
}

template <class H, int G>
static int launch_residual(const spk_plan *P, const int *rp, const int *ci, const void *a, const void *x, const void *b,
                           void *r, int nrhs, int want_b, double *norms, cudaStream_t st)
{
    const long long warps = ((long long)P->n + (32 / G) - 1) / (32 / G);
    long long blocks = (warps * 32 + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    for (int h0 = 0; h0 < nrhs; h0 += RES_MAXH) {
        const int nr = nrhs - h0 < RES_MAXH ? nrhs - h0 : RES_MAXH;
        k_residual<H, G><<<(unsigned)blocks, 256, 0, st>>>(P->n, rp, ci, (const H *)a, (const H *)x, (const H *)b,
                                                          (H *)r, h0, nr, want_b, norms, nrhs);
        if (cudaGetLastError() != cudaSuccess) return SPK_ECUDA;
        ((spk_plan *)P)->launches++;
    }
    return SPK_OK;
}

template <class H>
static int residual_g(const spk_plan *P, const int *rp, const int *ci, const void *a, const void *x, const void *b,
                      void *r, int nrhs, int want_b, double *norms, cudaStream_t st)
{
    // few lanes per row: every shuffle step of the row reduction is an FP64
    // add per lane, and GB300's FP64 pipe is the residual's bottleneck
    const double per_row = P->n > 0 ? (double)P->nnz / P->n : 1.0;
    if (per_row >= 32) return launch_residual<H, 8>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
    if (per_row >= 8) return launch_residual<H, 4>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
    return launch_residual<H, 2>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
}

extern "C" int spk_residual(const spk_plan *P, const int *d_rowptr, const int *d_colind, const void *d_aij,
                            const void *d_x, const void *d_b, void *d_r, int nrhs, int want_bnorm, double *d_norms,
                            void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (ck(cudaMemsetAsync(d_norms, 0, sizeof(double) * 2 * nrhs, st))) return SPK_ECUDA;
    if (P->is_complex)
        return residual_g<cdouble>(P, d_rowptr, d_colind, d_aij, d_x, d_b, d_r, nrhs, want_bnorm, d_norms, st);
    return residual_g<double>(P, d_rowptr, d_colind, d_aij, d_x, d_b, d_r, nrhs, want_bnorm, d_norms, st);
}

// ------------------------------------------------------------ phase timing
extern "C" void spk_phase_begin(spk_plan *P, int phase, void *stream)
{
    if (!P->timing) return;
    if (!P->ev) {
        cudaEvent_t *ev = (cudaEvent_t *)calloc(2 * SPK_MAX_EVENTS, sizeof(cudaEvent_t));
        if (!ev) return;
        for (int i = 0; i < 2 * SPK_MAX_EVENTS; i++) cudaEventCreate(&ev[i]);
        P->ev = ev;
        P->nev = 0;
    }
    if (P->nev >= SPK_MAX_EVENTS) spk_phase_collect(P);
    cudaEvent_t *ev = (cudaEvent_t *)P->ev;
    P->ev_phase[P->nev] = phase;
    cudaEventRecord(ev[2 * P->nev], (cudaStream_t)stream);
}
extern "C" void spk_phase_end(spk_plan *P, void *stream)
{
    if (!P->timing || !P->ev) return;
    cudaEvent_t *ev = (cudaEvent_t *)P->ev;
    cudaEventRecord(ev[2 * P->nev + 1], (cudaStream_t)stream);
    P->nev++;
}
extern "C" int spk_phase_collect(spk_plan *P)
{
    if (!P->ev) return SPK_OK;
    cudaEvent_t *ev = (cudaEvent_t *)P->ev;
    for (int i = 0; i < P->nev; i++) {
        float ms = 0.f;
        if (cudaEventSynchronize(ev[2 * i + 1]) != cudaSuccess) return SPK_ECUDA;
        if (cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]) != cudaSuccess) return SPK_ECUDA;
        P->phase_ms[P->ev_phase[i]] += ms;
        P->phase_calls[P->ev_phase[i]]++;
    }
    P->nev = 0;
    return SPK_OK;
}
extern "C" void spk_phase_destroy(spk_plan *P)
{
    if (!P->ev) return;
    cudaEvent_t *ev = (cudaEvent_t *)P->ev;
    for (int i = 0; i < 2 * SPK_MAX_EVENTS; i++) cudaEventDestroy(ev[i]);
    free(ev);
    P->ev = NULL;
}
