// spike_util.cu -- device plumbing, CSR analysis and the FP64 residual.
//
//   k_analyze    bandwidth (matrix_ComputeBandwidth, OpenMP/spike_algebra.c
//                :56-95) plus CSR validation in one streaming pass over colind: rowptr
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
extern "C" int spk_set_device(int dev) { return ck(cudaSetDevice(dev)); }
extern "C" int spk_mem_info(size_t *free_b, size_t *total_b)
{
    *free_b = *total_b = 0;
    return ck(cudaMemGetInfo(free_b, total_b));
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
// Stream-ordered allocation (stream != NULL): no device-wide synchronisation,
// so contexts on different streams keep overlapping while they allocate.  The
// device's default pool keeps freed memory for reuse (release threshold raised
// once per device).
extern "C" int spk_malloc_on(void **p, size_t bytes, void *stream)
{
    if (!stream) return spk_malloc(p, bytes);
    *p = nullptr;
    if (bytes == 0) bytes = 256;
    static int pool_dev[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && !pool_dev[dev]) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            unsigned long long thr = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        pool_dev[dev] = 1;
    }
    cudaError_t e = cudaMallocAsync(p, bytes, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_last_cuda = e;
        cudaGetLastError();
        *p = nullptr;
        return SPK_EMEM;
    }
    return SPK_OK;
}
extern "C" void spk_free_on(void *p, void *stream)
{
    if (!p) return;
    if (stream)
        cudaFreeAsync(p, (cudaStream_t)stream);
    else
        cudaFree(p);
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
// height rows of width bytes each, rows dpitch / spitch bytes apart, either
// direction (the pointers say which)
extern "C" int spk_memcpy_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                             void *stream)
{
    if (!width || !height) return SPK_OK;
    return ck(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, cudaMemcpyDefault, (cudaStream_t)stream));
}
// page-locked host memory (staging that is copied to and from the device)
extern "C" int spk_host_alloc(void **p, size_t bytes)
{
    *p = nullptr;
    cudaError_t e = cudaMallocHost(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        g_last_cuda = e;
        cudaGetLastError();
        *p = nullptr;
        return SPK_EMEM;
    }
    return SPK_OK;
}
extern "C" void spk_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}
extern "C" int spk_memset(void *dst, int v, size_t bytes, void *stream)
{
    return ck(cudaMemsetAsync(dst, v, bytes, (cudaStream_t)stream));
}

// ------------------------------------------------------------ analysis
// Each warp takes a chunk of AN_ROWS rows and streams their entries as one
// contiguous range (coalesced); a lane tracks the row of its entries by
// advancing through the chunk's row pointers.  A chunk whose row pointers are
// out of range or decreasing is flagged and not scanned.
constexpr int AN_ROWS = 64;
__global__ void k_analyze(int n, long long nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
                          int *out)
{
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    int ku = 0, kl = 0;
    unsigned flags = 0;
    for (long long r0 = warp * AN_ROWS; r0 < n; r0 += nwarps * AN_ROWS) {
        const long long r1 = min((long long)n, r0 + AN_ROWS);
        bool bad = false;
        for (long long r = r0 + lane; r < r1; r += 32) {
            const long long t0 = rowptr[r], t1 = rowptr[r + 1];
            if (t0 < 0 || t1 > nnz || t1 < t0) bad = true;
        }
        if (__any_sync(0xffffffffu, bad)) {
            flags |= SPK_DEV_ERR_CSR;
            continue;
        }
        const long long tb = rowptr[r0], te = rowptr[r1];
        long long row = r0;
        // four 32-entry pieces per iteration, their loads issued together; an
        // entry's predecessor is read directly (an L1 hit), so iterations do
        // not wait on one another
        for (long long base = tb; base < te; base += 128) {
            int c[4], pc[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const long long t = base + 32 * u + lane;
                c[u] = t < te ? colind[t] : 0;
                pc[u] = (t < te && t > tb) ? colind[t - 1] : 0;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const long long t = base + 32 * u + lane;
                if (t >= te) continue;
                while (rowptr[row + 1] <= t) row++; // stops by r1: t < rowptr[r1]
                if (c[u] < 0 || c[u] >= n) {
                    flags |= SPK_DEV_ERR_CSR;
                    continue;
                }
                if (t > rowptr[row] && pc[u] >= c[u]) flags |= SPK_DEV_ERR_CSR;
                ku = max(ku, c[u] - (int)row);
                kl = max(kl, (int)row - c[u]);
            }
        }
    }
    if (warp == 0 && lane == 0 && (rowptr[0] != 0 || rowptr[n] != nnz)) flags |= SPK_DEV_ERR_CSR;
    for (int o = 16; o > 0; o >>= 1) {
        ku = max(ku, __shfl_xor_sync(0xffffffffu, ku, o));
        kl = max(kl, __shfl_xor_sync(0xffffffffu, kl, o));
        flags |= __shfl_xor_sync(0xffffffffu, flags, o);
    }
    if (lane == 0) { // (read first: most warps have nothing larger to add)
        if (ku > *(volatile const int *)&out[0]) atomicMax(&out[0], ku);
        if (kl > *(volatile const int *)&out[1]) atomicMax(&out[1], kl);
        if (flags) atomicOr((unsigned *)&out[2], flags);
    }
}

extern "C" int spk_analyze(int n, long long nnz, const int *d_rowptr, const int *d_colind, int *d_out, int *out,
                           void *stream, long long *launches)
{
    cudaStream_t st = (cudaStream_t)stream;
    int r = ck(cudaMemsetAsync(d_out, 0, 4 * sizeof(int), st));
    if (r == SPK_OK && n > 0) {
        const long long warps_needed = (n + AN_ROWS - 1) / AN_ROWS;
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
// G lanes per row; NH columns per pass over a row's entries (the CSR entries
// are read once per pass, not once per column); per-column squared norms
// summed within each warp by shuffles, then once per warp in shared memory
// (contended FP64 shared atomics retry on the FP64 pipe), then once per CTA
// into norms[].
constexpr int RES_MAXH = 32;

template <class H, int G, int NH, bool IMPL>
__global__ void __launch_bounds__(256)
    k_residual(int n, const int *__restrict__ rowptr, const int *__restrict__ colind, const H *__restrict__ aij,
               const H *__restrict__ x, const H *__restrict__ b, H *r, int h0, int nr, int want_b, double *norms,
               int nrhs_total, int impl_kl)
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
    for (int hb = 0; hb < nr; hb += NH) {
        double lr[NH], lb[NH];
        const H *xj[NH]; // this pass's columns of x (a column past nr repeats the last one, unused)
#pragma unroll
        for (int j = 0; j < NH; j++) {
            lr[j] = lb[j] = 0.0;
            xj[j] = x + (size_t)(h0 + min(hb + j, nr - 1)) * n;
        }
        for (long long base = warp * RPW; base < n; base += nwarps * RPW) {
            const long long row = base + lane / G;
            const bool valid = row < n;
            const int t0 = valid ? rowptr[row] : 0, t1 = valid ? rowptr[row + 1] : 0;
            // IMPL: the row is the full band (checked on the host), colind is not read
            const int cfirst = IMPL ? max(0, (int)row - impl_kl) - t0 : 0;
            H acc[NH];
#pragma unroll
            for (int j = 0; j < NH; j++) acc[j] = sc_zero<H>();
            for (int t = t0 + sub; t < t1; t += G) {
                const H av = aij[t];
                const int c = IMPL ? cfirst + t : colind[t];
#pragma unroll
                for (int j = 0; j < NH; j++)
                    if (hb + j < nr) acc[j] = madd(acc[j], av, xj[j][c]);
            }
#pragma unroll
            for (int j = 0; j < NH; j++)
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    if constexpr (sizeof(H) == 8) {
                        acc[j] = acc[j] + __shfl_xor_sync(0xffffffffu, acc[j], o);
                    } else {
                        H other;
                        other.re = __shfl_xor_sync(0xffffffffu, acc[j].re, o);
                        other.im = __shfl_xor_sync(0xffffffffu, acc[j].im, o);
                        acc[j] = acc[j] + other;
                    }
                }
            if (sub == 0 && valid) {
#pragma unroll
                for (int j = 0; j < NH; j++) {
                    if (hb + j >= nr) break;
                    const size_t off = (size_t)(h0 + hb + j) * n + row;
                    const H bv = b[off];
                    const H rv = bv - acc[j];
                    r[off] = rv;
                    lr[j] += sc_abs2(rv);
                    if (want_b) lb[j] += sc_abs2(bv);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NH; j++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lr[j] += __shfl_xor_sync(0xffffffffu, lr[j], o);
                lb[j] += __shfl_xor_sync(0xffffffffu, lb[j], o);
            }
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < NH; j++) {
                if (hb + j >= nr) break;
                atomicAdd(&sr[hb + j], lr[j]);
                if (want_b) atomicAdd(&sb[hb + j], lb[j]);
            }
    }
    __syncthreads();
    for (int h = threadIdx.x; h < nr; h += blockDim.x) {
        atomicAdd(&norms[h0 + h], sr[h]);
        if (want_b) atomicAdd(&norms[nrhs_total + h0 + h], sb[h]);
    }
}

template <class H, int G, bool IMPL>
static int launch_residual(const spk_plan *P, const int *rp, const int *ci, const void *a, const void *x, const void *b,
                           void *r, int nrhs, int want_b, double *norms, cudaStream_t st)
{
    const long long warps = ((long long)P->n + (32 / G) - 1) / (32 / G);
    long long blocks = (warps * 32 + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    for (int h0 = 0; h0 < nrhs; h0 += RES_MAXH) {
        const int nr = nrhs - h0 < RES_MAXH ? nrhs - h0 : RES_MAXH;
        if (nr >= 4)
            k_residual<H, G, 4, IMPL><<<(unsigned)blocks, 256, 0, st>>>(P->n, rp, ci, (const H *)a, (const H *)x,
                                                                 (const H *)b, (H *)r, h0, nr, want_b, norms, nrhs,
                                                                 P->impl_cols ? P->impl_kl : -1);
        else if (nr >= 2)
            k_residual<H, G, 2, IMPL><<<(unsigned)blocks, 256, 0, st>>>(P->n, rp, ci, (const H *)a, (const H *)x,
                                                                 (const H *)b, (H *)r, h0, nr, want_b, norms, nrhs,
                                                                 P->impl_cols ? P->impl_kl : -1);
        else
            k_residual<H, G, 1, IMPL><<<(unsigned)blocks, 256, 0, st>>>(P->n, rp, ci, (const H *)a, (const H *)x,
                                                                 (const H *)b, (H *)r, h0, nr, want_b, norms, nrhs,
                                                                 P->impl_cols ? P->impl_kl : -1);
        if (cudaGetLastError() != cudaSuccess) return SPK_ECUDA;
        ((spk_plan *)P)->launches++;
    }
    return SPK_OK;
}

// lanes per row of the residual: 4 for long rows with one column, 2 for long
// rows with several columns and for medium rows, 1 for short rows
static int res_lanes(double per_row, int nrhs)
{
    if (per_row >= 64) return nrhs == 1 ? 4 : 2;
    return per_row >= 12 ? 2 : 1;
}

template <class H>
static int residual_g(const spk_plan *P, const int *rp, const int *ci, const void *a, const void *x, const void *b,
                      void *r, int nrhs, int want_b, double *norms, cudaStream_t st)
{
    // few lanes per row: every shuffle step of the row reduction is an FP64
    // add per lane, and GB300's FP64 pipe is the residual's bottleneck
    const double per_row = P->n > 0 ? (double)P->nnz / P->n : 1.0;
    // one column: 4 lanes from 64 entries a row; several columns: 2 lanes (a
    // lane's multiply-adds per reduction step grow with the columns)
    const int g = res_lanes(per_row, nrhs);
    if (P->impl_cols) {
        if (g == 4) return launch_residual<H, 4, true>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
        if (g == 2) return launch_residual<H, 2, true>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
        return launch_residual<H, 1, true>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
    }
    if (g == 4) return launch_residual<H, 4, false>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
    if (g == 2) return launch_residual<H, 2, false>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
    return launch_residual<H, 1, false>(P, rp, ci, a, x, b, r, nrhs, want_b, norms, st);
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

// ------------------------------------------------------------ batch residual
// One CTA per chunk of rows of one system; G lanes per row; NH right-hand-side
// columns per pass over the row's entries (the CSR entries are read once per
// pass, not once per column).
template <class H, int G, int NH>
__global__ void __launch_bounds__(256)
    k_residual_batch(const spk_sysref *__restrict__ sys, const int2 *__restrict__ chunks, int R, long long n_rows,
                     int nrhs, int have_x, H *r, double *norms)
{
    __shared__ double sr[NH], sb[NH];
    if (threadIdx.x < NH) sr[threadIdx.x] = sb[threadIdx.x] = 0.0;
    const int2 ch = chunks[blockIdx.x];
    const spk_sysref S = sys[ch.x];
    const int n = S.n, lr0 = ch.y, lr1 = min(n, ch.y + R);
    const H *__restrict__ a = (const H *)S.aij;
    const H *__restrict__ x = (const H *)S.x;
    const H *__restrict__ b = (const H *)S.b;
    const int sub = threadIdx.x % G;
    constexpr int RPB = 256 / G; // rows per CTA per pass
    for (int h0 = 0; h0 < nrhs; h0 += NH) {
        double lr[NH], lb[NH];
        const H *xj[NH]; // column pointers, hoisted out of the entry loop (no 64-bit offset per entry)
#pragma unroll
        for (int j = 0; j < NH; j++) {
            lr[j] = lb[j] = 0.0;
            xj[j] = x + (size_t)(h0 + j < nrhs ? h0 + j : h0) * n;
        }
        __syncthreads();
        // every lane runs every iteration so the shuffles see the full warp
        for (int base = lr0; base < lr1; base += RPB) {
            const int row = base + threadIdx.x / G;
            const bool valid = row < lr1;
            H acc[NH];
#pragma unroll
            for (int j = 0; j < NH; j++) acc[j] = sc_zero<H>();
            if (have_x && valid) {
                const int t0 = S.rowptr[row], t1 = S.rowptr[row + 1];
                for (int t = t0 + sub; t < t1; t += G) {
                    const H av = a[t];
                    const int c = S.colind[t];
#pragma unroll
                    for (int j = 0; j < NH; j++)
                        if (h0 + j < nrhs) acc[j] = madd(acc[j], av, xj[j][c]);
                }
            }
#pragma unroll
            for (int j = 0; j < NH; j++)
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    if constexpr (sizeof(H) == 8) {
                        acc[j] = acc[j] + __shfl_xor_sync(0xffffffffu, acc[j], o);
                    } else {
                        H other;
                        other.re = __shfl_xor_sync(0xffffffffu, acc[j].re, o);
                        other.im = __shfl_xor_sync(0xffffffffu, acc[j].im, o);
                        acc[j] = acc[j] + other;
                    }
                }
            if (sub == 0 && valid) {
#pragma unroll
                for (int j = 0; j < NH; j++) {
                    if (h0 + j >= nrhs) break;
                    const H bv = b[(size_t)(h0 + j) * n + row];
                    const H rv = bv - acc[j];
                    r[(size_t)(h0 + j) * n_rows + S.row0 + row] = rv;
                    lr[j] += sc_abs2(rv);
                    lb[j] += sc_abs2(bv);
                }
            }
        }
        // warp sums first: one shared atomic per warp and column
#pragma unroll
        for (int j = 0; j < NH; j++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lr[j] += __shfl_xor_sync(0xffffffffu, lr[j], o);
                lb[j] += __shfl_xor_sync(0xffffffffu, lb[j], o);
            }
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int j = 0; j < NH; j++) {
                if (h0 + j >= nrhs) break;
                atomicAdd(&sr[j], lr[j]);
                atomicAdd(&sb[j], lb[j]);
            }
        __syncthreads();
        if (threadIdx.x < NH && h0 + (int)threadIdx.x < nrhs) {
            double *ns = norms + (size_t)ch.x * 2 * nrhs;
            atomicAdd(&ns[h0 + threadIdx.x], sr[threadIdx.x]);
            atomicAdd(&ns[nrhs + h0 + threadIdx.x], sb[threadIdx.x]);
            sr[threadIdx.x] = sb[threadIdx.x] = 0.0;
        }
    }
}

template <class H, int G>
static int residual_batch_g(const spk_sysref *d_sys, const int *d_chunks, int nchunks, int R, long long n_rows,
                            int nrhs, int have_x, void *d_r, double *d_norms, cudaStream_t st)
{
    const int2 *ch = (const int2 *)d_chunks;
    if (nrhs >= 4)
        k_residual_batch<H, G, 4><<<nchunks, 256, 0, st>>>(d_sys, ch, R, n_rows, nrhs, have_x, (H *)d_r, d_norms);
    else if (nrhs >= 2)
        k_residual_batch<H, G, 2><<<nchunks, 256, 0, st>>>(d_sys, ch, R, n_rows, nrhs, have_x, (H *)d_r, d_norms);
    else
        k_residual_batch<H, G, 1><<<nchunks, 256, 0, st>>>(d_sys, ch, R, n_rows, nrhs, have_x, (H *)d_r, d_norms);
    return ck(cudaGetLastError());
}

extern "C" int spk_residual_batch(const spk_sysref *d_sys, const int *d_chunks, int nchunks, int rows_per_chunk,
                                  int row_len, long long n_rows, int nrhs, int is_complex, int have_x, void *d_r,
                                  double *d_norms, void *stream, long long *launches)
{
    if (nchunks <= 0) return SPK_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (launches) (*launches)++;
    const int R = rows_per_chunk;
    // lanes per row from the rows' length (as in the single-system residual)
    if (is_complex) {
        if (res_lanes(row_len, nrhs) == 4) return residual_batch_g<cdouble, 4>(d_sys, d_chunks, nchunks, R, n_rows, nrhs, have_x, d_r, d_norms, st);
        if (res_lanes(row_len, nrhs) == 2) return residual_batch_g<cdouble, 2>(d_sys, d_chunks, nchunks, R, n_rows, nrhs, have_x, d_r, d_norms, st);
        return residual_batch_g<cdouble, 1>(d_sys, d_chunks, nchunks, R, n_rows, nrhs, have_x, d_r, d_norms, st);
    }
    if (res_lanes(row_len, nrhs) == 4) return residual_batch_g<double, 4>(d_sys, d_chunks, nchunks, R, n_rows, nrhs, have_x, d_r, d_norms, st);
    if (res_lanes(row_len, nrhs) == 2) return residual_batch_g<double, 2>(d_sys, d_chunks, nchunks, R, n_rows, nrhs, have_x, d_r, d_norms, st);
    return residual_batch_g<double, 1>(d_sys, d_chunks, nchunks, R, n_rows, nrhs, have_x, d_r, d_norms, st);
}

__global__ void k_batch_relres(const double *__restrict__ norms, int nsys, int nrhs, double *relres,
                               unsigned long long *worst)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const double *ns = norms + (size_t)s * 2 * nrhs;
    double w = 0.0;
    for (int h = 0; h < nrhs; h++) {
        const double bn = sqrt(ns[nrhs + h]);
        const double v = sqrt(ns[h]) / (bn > 0.0 ? bn : 1.0);
        if (!(v <= w)) w = v; // NaN propagates
    }
    relres[s] = w;
    // non-negative doubles (and NaN above +inf) order like their bit patterns
    atomicMax(worst, (unsigned long long)__double_as_longlong(w));
}

extern "C" int spk_batch_relres(const double *d_norms, int nsys, int nrhs, double *d_relres,
                                unsigned long long *d_worst, void *stream, long long *launches)
{
    if (nsys <= 0) return SPK_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (ck(cudaMemsetAsync(d_worst, 0, sizeof(unsigned long long), st))) return SPK_ECUDA;
    k_batch_relres<<<(nsys + 255) / 256, 256, 0, st>>>(d_norms, nsys, nrhs, d_relres, d_worst);
    if (launches) (*launches)++;
    return ck(cudaGetLastError());
}

// ------------------------------------------------------------ graphs, fork/join, timers
extern "C" int spk_capture_begin(void *stream)
{
    return ck(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
}
extern "C" int spk_capture_end(void *stream, void **graph_exec)
{
    *graph_exec = nullptr;
    cudaGraph_t g = nullptr;
    if (ck(cudaStreamEndCapture((cudaStream_t)stream, &g))) return SPK_ECUDA;
    cudaGraphExec_t e = nullptr;
    const int r = ck(cudaGraphInstantiate(&e, g, 0));
    cudaGraphDestroy(g);
    if (r != SPK_OK) return r;
    *graph_exec = (void *)e;
    return SPK_OK;
}
extern "C" int spk_graph_launch(void *graph_exec, void *stream)
{
    return ck(cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream));
}
extern "C" void spk_graph_destroy(void *graph_exec)
{
    if (graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)graph_exec);
}
extern "C" int spk_event_create(void **event)
{
    cudaEvent_t e;
    const int r = ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    *event = r == SPK_OK ? (void *)e : nullptr;
    return r;
}
extern "C" void spk_event_destroy(void *event)
{
    if (event) cudaEventDestroy((cudaEvent_t)event);
}
extern "C" int spk_event_record(void *event, void *stream)
{
    return ck(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream));
}
extern "C" int spk_stream_wait_event(void *stream, void *event)
{
    return ck(cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)event, 0));
}
extern "C" int spk_stream_fork(void *parent, void *child)
{
    cudaEvent_t e;
    if (ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return SPK_ECUDA;
    int r = ck(cudaEventRecord(e, (cudaStream_t)parent));
    if (r == SPK_OK) r = ck(cudaStreamWaitEvent((cudaStream_t)child, e, 0));
    cudaEventDestroy(e);
    return r;
}
extern "C" int spk_timer_begin(void **timer, void *stream)
{
    cudaEvent_t *ev = (cudaEvent_t *)calloc(2, sizeof(cudaEvent_t));
    *timer = nullptr;
    if (!ev) return SPK_EMEM;
    if (ck(cudaEventCreate(&ev[0])) || ck(cudaEventCreate(&ev[1]))) {
        free(ev);
        return SPK_ECUDA;
    }
    *timer = ev;
    return ck(cudaEventRecord(ev[0], (cudaStream_t)stream));
}
extern "C" int spk_timer_end(void *timer, void *stream, double *ms)
{
    cudaEvent_t *ev = (cudaEvent_t *)timer;
    float f = 0.f;
    int r = ck(cudaEventRecord(ev[1], (cudaStream_t)stream));
    if (r == SPK_OK) r = ck(cudaEventSynchronize(ev[1]));
    if (r == SPK_OK) r = ck(cudaEventElapsedTime(&f, ev[0], ev[1]));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    free(ev);
    *ms = f;
    return r;
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

// ------------------------------------------------------------ sharded solve: a rank's rows
// Bandwidth of rows [row0, row0 + m) of a matrix whose entries carry GLOBAL
// column indices (rowptr from 0): out[0] = max(c - row), out[1] = max(row - c),
// out[2] = 1 if a row pointer or column is out of range.  Grid-stride over
// entries; a row per thread with its entries.
__global__ void k_rows_band(int m, long long nnz, int row0, int n, const int *__restrict__ rowptr,
                            const int *__restrict__ colind, int *out)
{
    int ku = 0, kl = 0, bad = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const int t0 = rowptr[r], t1 = rowptr[r + 1];
        if (t0 < 0 || t1 < t0 || (long long)t1 > nnz) {
            bad = 1;
            continue;
        }
        for (int t = t0; t < t1; t++) {
            const int c = colind[t];
            if (c < 0 || c >= n) bad = 1;
            ku = max(ku, c - (row0 + r));
            kl = max(kl, (row0 + r) - c);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        ku = max(ku, __shfl_xor_sync(0xffffffffu, ku, o));
        kl = max(kl, __shfl_xor_sync(0xffffffffu, kl, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, ku);
        atomicMax(out + 1, kl);
        if (bad) atomicOr(out + 2, 1);
    }
}

extern "C" int spk_rows_band(int m, long long nnz, int row0, int n, const int *d_rowptr, const int *d_colind,
                             int *d_out, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    int r = ck(cudaMemsetAsync(d_out, 0, 4 * sizeof(int), st));
    if (r == SPK_OK && m > 0) {
        long long blocks = ((long long)m + 255) / 256;
        if (blocks > 152 * 8) blocks = 152 * 8;
        k_rows_band<<<(unsigned)blocks, 256, 0, st>>>(m, nnz, row0, n, d_rowptr, d_colind, d_out);
        r = ck(cudaGetLastError());
    }
    return r;
}

// The local system of a sharded solve, in place: the rank's rows (rowptr from
// 0, global columns, values) were copied to rows [h, h + m) of rowptr and to
// entries [h, h + nnz) of colind / aij.  Shifts those row pointers by h and
// columns by h - row0, and writes h identity rows before and after.
__global__ void k_shard_local(int m, long long nnz, int h, int row0, int *rowptr, int *colind, double *aij)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long i = tid; i < h; i += stride) {
        rowptr[i] = (int)i;
        colind[i] = (int)i;
        aij[i] = 1.0;
        rowptr[h + m + 1 + i] = (int)(h + nnz + 1 + i);
        colind[h + nnz + i] = (int)(h + m + i);
        aij[h + nnz + i] = 1.0;
    }
    for (long long r = tid; r <= m; r += stride) rowptr[h + r] += h;
    for (long long t = tid; t < nnz; t += stride) colind[h + t] += h - row0;
}

extern "C" int spk_shard_local(int m, long long nnz, int h, int row0, int *d_rowptr, int *d_colind, double *d_aij,
                               void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    long long blocks = (nnz + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_shard_local<<<(unsigned)blocks, 256, 0, st>>>(m, nnz, h, row0, d_rowptr, d_colind, d_aij);
    return ck(cudaGetLastError());
}
