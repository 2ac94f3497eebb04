// spike_apply.cu -- right-hand-side phases of the SPIKE solve on sm_103a.
//
//   k_apply      y_i = A_i^{-1} r_i with the resident block factors: forward
//                z_J = r_J - L_J z_{J-1}, backward y_J = G_J (z_J - E_J y_{J+1}).
//                Replaces the reference's per-partition directSolver_SolveForRHS
//                on f_i (OpenMP/spike_interfaces.c:143) -- SuperLU dgstrs +
//                dgsrfs per column (OpenMP/spike_superlu.c:986,1002).
//                Two-sided partitions: k_tw_apply_fwd / mid / bwd (CTA per chain),
//                k_tw_apply_fwd_w / bwd_w (FP32 32-row tiles, one warp per chain),
//                k_qtw_apply_* (KB <= 4 on lanes); one-sided small bands on
//                lanes: k_quad_apply (KB <= 8).
//   k_ytips      bottom / top tips of y into the reduced right-hand side
//                (block_AddTipTOReducedRHS, OpenMP/spike_matrix.c:1272-1297).
//   k_retrieve   x_i (+)= y_i - V_i t_{i+1} - W_i b_{i-1} with the stored spikes
//                (k_retrieve_rows for KB 8..32, k_retrieve_rc for KB <= 4).
//                The reference re-factors A_i and re-solves
//                A_i x_i = f_i - B_i x_t - C_i x_b (OpenMP/spike_interfaces.c
//                :259-396); with the spikes resident this is one parallel pass.
#include "spike_common.cuh"

#include <algorithm>
#include <type_traits>

namespace {

constexpr int RC = 32;      // right-hand-side columns per CTA
constexpr int RCS = RC + 1; // row stride of the shared [KB][RC] vectors (odd: column-wise writes spread over banks)

// out[r][h] = sign * sum_k M[r][k] v[k][h] (+ base[r][h]), r < KB, h < nr.
// Mt: shared tile holding M transposed (the factor tiles are column-major in
// global memory); v, base, out: shared [KB][RC] vectors with row stride RCS.
// Four or more columns: each thread accumulates a 4 x 4 block (4 rows of M
// by one 16-byte load, 4 columns of v) over a slice of k, so a step moves
// 0.5 shared-memory words per FMA instead of 2; the k slices of a block are
// summed by shuffles.  Fewer columns: one output per lane group, k split
// across the group.
template <class T, int KB, bool HAS_BASE, int S = RCS>
__device__ void tile_mv(T *out, const T *Mt, const T *v, const T *base, int nr, bool negate)
{
    constexpr int NT = NTOf<KB>::value;
    constexpr int LD = TileLD<T, KB>::value;
    // (FP32 arithmetic only: the shuffle sums of the k slices would add FP64
    // work on GB300's slow FP64 pipe; and only where most threads stay busy)
    if constexpr (KB >= 8 && (std::is_same<T, float>::value || std::is_same<T, cfloat>::value)) {
      constexpr int RG = KB / 4; // row groups
      const int CG = (nr + 3) / 4;
      if (nr >= 4 && RG * CG * (RG < 8 ? RG : 8) >= NT / 2) {
        const int units = RG * CG;
        int spl = 1;
        while (spl < 8 && spl * 2 * units <= NT && spl * 2 <= RG) spl *= 2;
        const int tid = threadIdx.x;
        const int part = tid & (spl - 1);
        const int groups = NT / spl;
        const int iters = (units + groups - 1) / groups;
        for (int it = 0; it < iters; it++) {
            const int u = it * groups + tid / spl;
            const bool valid = u < units;
            const int uu = valid ? u : 0;
            const int r0 = (uu % RG) * 4, h0 = (uu / RG) * 4;
            T acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[i][c] = sc_zero<T>();
            for (int k = part; k < KB; k += spl) {
                T m[4], w[4];
                vld<T, 4>(m, Mt + k * LD + r0);
#pragma unroll
                for (int c = 0; c < 4; c++) w[c] = h0 + c < nr ? v[k * S + h0 + c] : sc_zero<T>();
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[i][c] = madd(acc[i][c], m[i], w[c]);
            }
            for (int off = spl >> 1; off > 0; off >>= 1)
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[i][c] = acc[i][c] + shfl_xor_any(acc[i][c], off);
            if (valid && part == 0) {
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int c = 0; c < 4; c++)
                        if (h0 + c < nr) {
                            const int q = (r0 + i) * S + h0 + c;
                            T val = negate ? -acc[i][c] : acc[i][c];
                            if (HAS_BASE) val = base[q] + val;
                            out[q] = val;
                        }
            }
        }
        return;
      }
    }
    // One column: a thread takes 4 rows (one 16-byte load per k) over an
    // interleaved slice of k, and the SL slices of a row group are summed by
    // one grouped transpose sum.
    if constexpr (KB >= 16) {
        constexpr int RG = KB / 4, SL = NT / RG, KS = KB / SL;
        static_assert(SL >= 4 && SL <= 32 && KS * SL == KB, "one-column slices");
        if (nr == 1) {
            const int lane = threadIdx.x & 31, slice = threadIdx.x & (SL - 1), r0 = (threadIdx.x / SL) * 4;
            T acc[4];
#pragma unroll
            for (int i = 0; i < 4; i++) acc[i] = sc_zero<T>();
#pragma unroll
            for (int kk = 0; kk < KS; kk++) {
                const int k = kk * SL + slice;
                T m[4];
                vld<T, 4>(m, Mt + k * LD + r0);
                const T x = v[k * S];
#pragma unroll
                for (int i = 0; i < 4; i++) acc[i] = madd(acc[i], m[i], x);
            }
            const T sum = warp_tsum<T, 4, SL>(acc, lane);
            constexpr int SH = (SL == 4 ? 2 : SL == 8 ? 3 : SL == 16 ? 4 : 5) - 2;
            if ((slice & ((1 << SH) - 1)) == 0) {
                const int r = r0 + (slice >> SH);
                T val = negate ? -sum : sum;
                if (HAS_BASE) val = base[r * S] + val;
                out[r * S] = val;
            }
            return;
        }
    }
    const int O = KB * nr;
    int spl = 1;
    while (spl < 32 && spl * 2 * O <= NT && spl * 2 <= KB) spl *= 2;
    const int tid = threadIdx.x;
    const int part = tid & (spl - 1);
    const int groups = NT / spl;
    // every thread runs the same number of iterations so the shuffles converge
    const int iters = (O + groups - 1) / groups;
    for (int it = 0; it < iters; it++) {
        const int o = it * groups + tid / spl;
        T acc = sc_zero<T>();
        int r = 0, h = 0;
        if (o < O) {
            r = o / nr;
            h = o - r * nr;
            for (int k = part; k < KB; k += spl) acc = madd(acc, Mt[k * LD + r], v[k * S + h]);
        }
        for (int off = spl >> 1; off > 0; off >>= 1) {
            if constexpr (sizeof(T) == 4) {
                acc = acc + __shfl_xor_sync(0xffffffffu, acc, off);
            } else {
                // generic path: shuffle the raw words
                T other;
                const unsigned *src = (const unsigned *)&acc;
                unsigned *dst = (unsigned *)&other;
#pragma unroll
                for (int w = 0; w < (int)(sizeof(T) / 4); w++) dst[w] = __shfl_xor_sync(0xffffffffu, src[w], off);
                acc = acc + other;
                continue;
            }
        }
        if (o < O && part == 0) {
            T val = negate ? -acc : acc;
            if (HAS_BASE) val = base[r * S + h] + val;
            out[r * S + h] = val;
        }
    }
}

// Right-hand-side rows of block J (FP64 -> factor precision) into registers.
// Vector elements q < KB * nr of block J: column h = q / KB, row lr = q % KB,
// so consecutive threads touch consecutive rows of one column (coalesced
// global accesses) and only the live columns are fetched.
template <class T, class H, int KB, int VPT>
__device__ __forceinline__ void fetch_r(T (&nxt)[VPT], const H *__restrict__ r, int n, int s, int m, int h0, int nr,
                                        int J)
{
    constexpr int NT = NTOf<KB>::value;
#pragma unroll
    for (int v = 0; v < VPT; v++) {
        const int q = threadIdx.x + v * NT;
        if (q < KB * nr) {
            const int h = q / KB, lr = q - h * KB, lrow = J * KB + lr;
            nxt[v] = lrow < m ? cvt_fast<T, H>(r[(size_t)(h0 + h) * n + s + lrow]) : sc_zero<T>();
        }
    }
}
// forward-sweep vector of block J into registers
template <class T, int KB, int VPT>
__device__ __forceinline__ void fetch_z(T (&nxt)[VPT], const T *gz, long long NP, long long rb, int h0, int nr, int J)
{
    constexpr int NT = NTOf<KB>::value;
#pragma unroll
    for (int v = 0; v < VPT; v++) {
        const int q = threadIdx.x + v * NT;
        if (q < KB * nr) {
            const int h = q / KB, lr = q - h * KB;
            nxt[v] = gz[(size_t)(h0 + h) * NP + rb + J * KB + lr];
        }
    }
}
template <class T, int KB, int VPT, int S = RCS> __device__ __forceinline__ void put_v(const T (&nxt)[VPT], T *sv, int nr)
{
    constexpr int NT = NTOf<KB>::value;
#pragma unroll
    for (int v = 0; v < VPT; v++) {
        const int q = threadIdx.x + v * NT;
        if (q < KB * nr) {
            const int h = q / KB, lr = q - h * KB;
            sv[lr * S + h] = nxt[v];
        }
    }
}

template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_apply(const int *__restrict__ part_start, const int *__restrict__ blk_off, const T *__restrict__ gL,
            const T *__restrict__ gG, const T *__restrict__ gE, const typename HighOf<T>::type *__restrict__ r,
            int n, int nrhs, long long NP, T *gz, T *gy)
{
    using H = typename HighOf<T>::type;
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int LDT = TileLD<T, KB>::value;
    constexpr int VPT = (KB * RC + NT - 1) / NT; // vector elements per thread
    const int part = blockIdx.x;
    const int h0 = blockIdx.y * RC;
    const int nr = min(RC, nrhs - h0);
    const int s = part_start[part], m = part_start[part + 1] - s;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    const long long rb = (long long)blk_off[part] * KB; // padded-row base

    // 128-row tiles (66 KB each in FP32) leave room for two tile buffers, not four
    constexpr int NB = KB >= 128 ? 1 : 2; // backward: buffers per tile kind
    constexpr int RD = 2 * NB;            // forward: ring depth
    extern __shared__ char smraw[];
    // backward buffers, selected by block parity when double: M tiles (G) then E tiles
    T *const sM0 = (T *)smem_align(smraw);
    T *const sE0 = sM0 + NB * KB * LDT;
#define SMA(par) (sM0 + ((par) & (NB - 1)) * KB * LDT)
#define SEA(par) (sE0 + ((par) & (NB - 1)) * KB * LDT)
    T *sv = sM0 + RD * KB * LDT; // [KB][RCS]
    T *sp = sv + KB * RCS;     // previous block's vector
    T *sw = sp + KB * RCS;     // work vector

    // the next block's right-hand-side rows ride in registers while the
    // current block computes; its tiles stream into the other buffer (cp.async)
    T nxt[VPT];
    // forward: z_J = r_J - L_J z_{J-1}.  It reads only L, so all the tile
    // buffers form a ring: L_{J+1..J+RD-1} stream in while block J computes.
#define RING(j) (sM0 + ((j) & (RD - 1)) * KB * LDT)
    for (int j = 1; j < RD; j++) {
        if (j < N) cp_async_tile<T, KB, NT>(RING(j), gL + tb + (size_t)j * TS);
        cp_async_commit();
    }
    fetch_r<T, H, KB, VPT>(nxt, r, n, s, m, h0, nr, 0);
    put_v<T, KB, VPT>(nxt, sv, nr);
    cp_async_wait_n<RD - 2>(); // L_1
    __syncthreads();
    for (int J = 0; J < N; J++) {
        if (J + RD - 1 < N) cp_async_tile<T, KB, NT>(RING(J + RD - 1), gL + tb + (size_t)(J + RD - 1) * TS);
        cp_async_commit();
        if (J + 1 < N) fetch_r<T, H, KB, VPT>(nxt, r, n, s, m, h0, nr, J + 1);
        if (J > 0)
            tile_mv<T, KB, true>(sw, RING(J), sp, sv, nr, true);
        else
            for (int q = threadIdx.x; q < KB * RCS; q += NT) sw[q] = sv[q];
        __syncthreads();
        for (int q = threadIdx.x; q < KB * nr; q += NT) {
            const int h = q / KB, lr = q - h * KB;
            const T v = sw[lr * RCS + h];
            sp[lr * RCS + h] = v;
            gz[(size_t)(h0 + h) * NP + rb + J * KB + lr] = v;
        }
        if (J + 1 < N) put_v<T, KB, VPT>(nxt, sv, nr);
        cp_async_wait_n<RD - 2>(); // L_{J+1}
        __syncthreads();
    }
#undef RING
    cp_async_wait_all();
    // backward: y_J = G_J (z_J - E_J y_{J+1})
    cp_async_tile<T, KB, NT>(SMA(N - 1), gG + tb + (N - 1) * TS);
    cp_async_commit();
    fetch_z<T, KB, VPT>(nxt, gz, NP, rb, h0, nr, N - 1);
    put_v<T, KB, VPT>(nxt, sv, nr);
    cp_async_wait_all();
    __syncthreads();
    for (int J = N - 1; J >= 0; J--) {
        if constexpr (NB == 1) { // single buffers: block J's tiles arrive now
            if (J < N - 1) {
                cp_async_tile<T, KB, NT>(SMA(J), gG + tb + J * TS);
                cp_async_tile<T, KB, NT>(SEA(J), gE + tb + J * TS);
                cp_async_commit();
                cp_async_wait_all();
                __syncthreads();
            }
        }
        if (J > 0) {
            if constexpr (NB == 2) {
                cp_async_tile<T, KB, NT>(SMA(J - 1), gG + tb + (J - 1) * TS);
                cp_async_tile<T, KB, NT>(SEA(J - 1), gE + tb + (J - 1) * TS);
                cp_async_commit();
            }
            fetch_z<T, KB, VPT>(nxt, gz, NP, rb, h0, nr, J - 1);
        }
        if (J < N - 1) {
            tile_mv<T, KB, true>(sw, SEA(J), sp, sv, nr, true);
            __syncthreads();
            tile_mv<T, KB, false>(sp, SMA(J), sw, nullptr, nr, false);
        } else {
            tile_mv<T, KB, false>(sp, SMA(J), sv, nullptr, nr, false);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < KB * nr; q += NT) {
            const int h = q / KB, lr = q - h * KB;
            gy[(size_t)(h0 + h) * NP + rb + J * KB + lr] = sp[lr * RCS + h];
        }
        if (J > 0) put_v<T, KB, VPT>(nxt, sv, nr);
        cp_async_wait_all();
        __syncthreads();
    }
}

#undef SMA
#undef SEA

// ------------------------------------------------------------ two-sided partitions
// y_i = A_i^{-1} r_i with the two-sided factors of spike_twist.cu (layout
// there): both halves sweep towards the middle block M, M is solved, and both
// halves sweep back out.  Sixteen right-hand-side columns per CTA keep two
// tiles and three vectors within a quarter of the SM's shared memory.
constexpr int RC2 = 16;
constexpr int RCS2 = RC2 + 1;
template <class T, int KB> constexpr size_t tw_apply_smem()
{
    return 16 + sizeof(T) * (2 * KB * TileLD<T, KB>::value + 3 * KB * RCS2);
}

//   top     z_J = r_J - L_J z_{J-1},  J = 0..M-1
//   bottom  w_J = r_J - U_J w_{J+1},  J = N-1..M   (U_M in gE)
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value, 4)
    k_tw_apply_fwd(const int *__restrict__ part_start, const int *__restrict__ blk_off, const T *__restrict__ gL,
                   const T *__restrict__ gE, const typename HighOf<T>::type *__restrict__ r, int n, int nrhs,
                   long long NP, T *gz)
{
    using H = typename HighOf<T>::type;
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int LDT = TileLD<T, KB>::value;
    constexpr int VPT = (KB * RC2 + NT - 1) / NT;
    const int part = blockIdx.x;
    const bool top = blockIdx.y == 0;
    const int h0 = blockIdx.z * RC2, nr = min(RC2, nrhs - h0);
    const int s = part_start[part], m = part_start[part + 1] - s;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const long long rb = (long long)blk_off[part] * KB;
    const int cnt = top ? M : N - M;

    extern __shared__ char smraw[];
    T *const t0 = (T *)smem_align(smraw), *const t1 = t0 + KB * LDT;
    T *sv = t1 + KB * LDT, *sp = sv + KB * RCS2, *sw = sp + KB * RCS2;
    auto blk = [&](int i) { return top ? i : N - 1 - i; };
    auto slot = [&](int i) { return (i & 1) ? t1 : t0; };
    auto ctile = [&](int i) { // coupling tile of step i >= 1
        const int J = blk(i);
        return (!top && J == M ? gE : gL) + tb + (size_t)J * TS;
    };

    T nxt[VPT];
    fetch_r<T, H, KB, VPT>(nxt, r, n, s, m, h0, nr, blk(0));
    put_v<T, KB, VPT, RCS2>(nxt, sv, nr);
    __syncthreads();
    for (int i = 0; i < cnt; i++) {
        const int J = blk(i);
        if (i + 1 < cnt) cp_async_tile<T, KB, NT>(slot(i + 1), ctile(i + 1));
        cp_async_commit();
        if (i + 1 < cnt) fetch_r<T, H, KB, VPT>(nxt, r, n, s, m, h0, nr, blk(i + 1));
        if (i > 0)
            tile_mv<T, KB, true, RCS2>(sw, slot(i), sp, sv, nr, true);
        else
            for (int q = threadIdx.x; q < KB * RCS2; q += NT) sw[q] = sv[q];
        __syncthreads();
        for (int q = threadIdx.x; q < KB * nr; q += NT) {
            const int h = q / KB, lr = q - h * KB;
            const T v = sw[lr * RCS2 + h];
            sp[lr * RCS2 + h] = v;
            gz[(size_t)(h0 + h) * NP + rb + J * KB + lr] = v;
        }
        if (i + 1 < cnt) put_v<T, KB, VPT, RCS2>(nxt, sv, nr);
        cp_async_wait_all();
        __syncthreads();
    }
}

// block M: z_M = w_M - L_M z_{M-1},  y_M = G_M z_M
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_tw_apply_mid(const int *__restrict__ blk_off, const T *__restrict__ gL, const T *__restrict__ gG, int nrhs,
                   long long NP, const T *__restrict__ gz, T *gy)
{
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int LDT = TileLD<T, KB>::value;
    const int part = blockIdx.x;
    const int h0 = blockIdx.y * RC2, nr = min(RC2, nrhs - h0);
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const long long rb = (long long)blk_off[part] * KB;

    extern __shared__ char smraw[];
    T *const sT = (T *)smem_align(smraw), *const sT2 = sT + KB * LDT;
    T *sv = sT2 + KB * LDT, *sp = sv + KB * RCS2, *sw = sp + KB * RCS2;
    cp_async_tile<T, KB, NT>(sT, gL + tb + (size_t)M * TS);
    cp_async_tile<T, KB, NT>(sT2, gG + tb + (size_t)M * TS);
    cp_async_commit();
    for (int q = threadIdx.x; q < KB * nr; q += NT) {
        const int h = q / KB, lr = q - h * KB;
        sv[lr * RCS2 + h] = gz[(size_t)(h0 + h) * NP + rb + M * KB + lr];
        sp[lr * RCS2 + h] = gz[(size_t)(h0 + h) * NP + rb + (M - 1) * KB + lr];
    }
    cp_async_wait_all();
    __syncthreads();
    tile_mv<T, KB, true, RCS2>(sw, sT, sp, sv, nr, true);
    __syncthreads();
    tile_mv<T, KB, false, RCS2>(sp, sT2, sw, nullptr, nr, false);
    __syncthreads();
    for (int q = threadIdx.x; q < KB * nr; q += NT) {
        const int h = q / KB, lr = q - h * KB;
        gy[(size_t)(h0 + h) * NP + rb + M * KB + lr] = sp[lr * RCS2 + h];
    }
}

//   top     y_J = G_J (z_J - A(J,J+1) y_{J+1}),  J = M-1..0
//   bottom  y_J = H_J (w_J - A(J,J-1) y_{J-1}),  J = M+1..N-1
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value, 4)
    k_tw_apply_bwd(const int *__restrict__ blk_off, const T *__restrict__ gG, const T *__restrict__ gE, int nrhs,
                   long long NP, const T *__restrict__ gz, T *gy)
{
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int LDT = TileLD<T, KB>::value;
    constexpr int VPT = (KB * RC2 + NT - 1) / NT;
    const int part = blockIdx.x;
    const bool top = blockIdx.y == 0;
    const int h0 = blockIdx.z * RC2, nr = min(RC2, nrhs - h0);
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const long long rb = (long long)blk_off[part] * KB;
    const int cnt = top ? M : N - 1 - M;

    extern __shared__ char smraw[];
    T *const sG = (T *)smem_align(smraw), *const sE = sG + KB * LDT;
    T *sv = sE + KB * LDT, *sp = sv + KB * RCS2, *sw = sp + KB * RCS2;
    auto blk = [&](int i) { return top ? M - 1 - i : M + 1 + i; };

    T nxt[VPT];
    cp_async_tile<T, KB, NT>(sG, gG + tb + (size_t)blk(0) * TS);
    cp_async_tile<T, KB, NT>(sE, gE + tb + (size_t)blk(0) * TS);
    cp_async_commit();
    fetch_z<T, KB, VPT>(nxt, gz, NP, rb, h0, nr, blk(0));
    put_v<T, KB, VPT, RCS2>(nxt, sv, nr);
    for (int q = threadIdx.x; q < KB * nr; q += NT) {
        const int h = q / KB, lr = q - h * KB;
        sp[lr * RCS2 + h] = gy[(size_t)(h0 + h) * NP + rb + M * KB + lr]; // y_M
    }
    cp_async_wait_all();
    __syncthreads();
    for (int i = 0; i < cnt; i++) {
        const int J = blk(i);
        const bool more = i + 1 < cnt;
        if (more) fetch_z<T, KB, VPT>(nxt, gz, NP, rb, h0, nr, blk(i + 1));
        tile_mv<T, KB, true, RCS2>(sw, sE, sp, sv, nr, true);
        __syncthreads();
        if (more) {
            cp_async_tile<T, KB, NT>(sE, gE + tb + (size_t)blk(i + 1) * TS);
            cp_async_commit();
        }
        tile_mv<T, KB, false, RCS2>(sp, sG, sw, nullptr, nr, false);
        __syncthreads();
        if (more) {
            cp_async_tile<T, KB, NT>(sG, gG + tb + (size_t)blk(i + 1) * TS);
            cp_async_commit();
        }
        for (int q = threadIdx.x; q < KB * nr; q += NT) {
            const int h = q / KB, lr = q - h * KB;
            gy[(size_t)(h0 + h) * NP + rb + J * KB + lr] = sp[lr * RCS2 + h];
        }
        if (more) put_v<T, KB, VPT, RCS2>(nxt, sv, nr);
        cp_async_wait_all();
        __syncthreads();
    }
}

// The two-sided sweeps for FP32 16- and 32-row tiles on KB lanes per
// (partition, half, chunk of HC columns) chain -- a warp at KB = 32, a
// half-warp at KB = 16 -- lane l of the chain owning row l of every block:
// the step's coupling tile arrives straight from global memory into
// registers (lane l reads row l of the column-major tile: consecutive
// addresses across the chain), one step ahead, and the previous block's
// vector is broadcast from a small shared buffer.  No CTA barrier (a chain's
// lanes synchronise among themselves): many chains share each SM, and a step
// is a few hundred instructions.  The middle block is k_tw_apply_mid's.
constexpr int TWW_CHAINS = 4; // warps per CTA of the one-warp sweeps

template <int KB> __device__ __forceinline__ unsigned tww_mask()
{
    return KB == 32 ? 0xffffffffu : (0xffffu << (threadIdx.x & 16));
}
template <class T, int KB> __device__ __forceinline__ void tww_row(T (&d)[KB], const T *g, int row)
{
#pragma unroll
    for (int k = 0; k < KB; k++) d[k] = g[(size_t)k * KB + row];
}
// out[h] (+|-)= sum_k M[row][k] v[k][h]; v: shared [KB][HC], read by broadcast
template <class T, int KB, int HC, bool SUB>
__device__ __forceinline__ void tww_mv(T (&out)[HC], const T (&m)[KB], const T *v)
{
#pragma unroll
    for (int k = 0; k < KB; k++) {
        T vk[HC];
        vld<T, HC>(vk, v + k * HC);
#pragma unroll
        for (int h = 0; h < HC; h++) out[h] = SUB ? msub(out[h], m[k], vk[h]) : madd(out[h], m[k], vk[h]);
    }
}

//   top     z_J = r_J - L_J z_{J-1},  J = 0..M-1
//   bottom  w_J = r_J - U_J w_{J+1},  J = N-1..M   (U_M in gE)
template <class T, int KB, int HC>
__global__ void __launch_bounds__(32 * TWW_CHAINS)
    k_tw_apply_fwd_w(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                     const T *__restrict__ gL, const T *__restrict__ gE, const typename HighOf<T>::type *__restrict__ r,
                     int n, int nrhs, long long NP, T *gz)
{
    static_assert(KB == 16 || KB == 32, "KB lanes per chain");
    constexpr int CPW = 32 / KB; // chains per warp
    constexpr size_t TS = (size_t)KB * KB;
    __shared__ __align__(16) T vs[TWW_CHAINS * CPW][KB * HC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row = lane % KB;
    const int slot = warp * CPW + lane / KB;
    const int nch = (nrhs + HC - 1) / HC;
    const long long chain = (long long)blockIdx.x * TWW_CHAINS * CPW + slot;
    if (chain >= (long long)p * 2 * nch) return; // the whole chain
    const unsigned msk = tww_mask<KB>();
    const int part = (int)(chain / (2 * nch)), rem = (int)(chain - (long long)part * 2 * nch);
    const bool top = (rem & 1) == 0;
    const int h0 = (rem >> 1) * HC, nr = min(HC, nrhs - h0);
    const int s = part_start[part], m = part_start[part + 1] - s;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const long long rb = (long long)blk_off[part] * KB;
    const int cnt = top ? M : N - M;
    T *vw = vs[slot];
    auto blk = [&](int i) { return top ? i : N - 1 - i; };
    auto ctile = [&](int i) {
        const int J = blk(i);
        return (!top && J == M ? gE : gL) + tb + (size_t)J * TS;
    };
    auto fetch = [&](T (&d)[HC], int i) {
        const int rw = blk(i) * KB + row;
#pragma unroll
        for (int h = 0; h < HC; h++)
            d[h] = (h < nr && rw < m) ? cvt_fast<T>(r[(size_t)(h0 + h) * n + s + rw]) : sc_zero<T>();
    };
    T rn[HC], mc[KB], mn[KB];
    fetch(rn, 0);
    if (cnt > 1) tww_row<T, KB>(mn, ctile(1), row);
    for (int i = 0; i < cnt; i++) {
        const int J = blk(i);
        T z[HC];
#pragma unroll
        for (int h = 0; h < HC; h++) z[h] = rn[h];
        if (i + 1 < cnt) fetch(rn, i + 1);
        if (i > 0) {
#pragma unroll
            for (int k = 0; k < KB; k++) mc[k] = mn[k];
            if (i + 1 < cnt) tww_row<T, KB>(mn, ctile(i + 1), row);
            tww_mv<T, KB, HC, true>(z, mc, vw);
        }
        __syncwarp(msk); // every lane of the chain has read the previous vector
        vst<T, HC>(vw + row * HC, z);
#pragma unroll
        for (int h = 0; h < HC; h++)
            if (h < nr) gz[(size_t)(h0 + h) * NP + rb + (size_t)J * KB + row] = z[h];
        __syncwarp(msk);
    }
}

//   top     y_J = G_J (z_J - A(J,J+1) y_{J+1}),  J = M-1..0
//   bottom  y_J = H_J (w_J - A(J,J-1) y_{J-1}),  J = M+1..N-1
template <class T, int KB, int HC>
__global__ void __launch_bounds__(32 * TWW_CHAINS)
    k_tw_apply_bwd_w(const int *__restrict__ blk_off, int p, const T *__restrict__ gG, const T *__restrict__ gE,
                     int nrhs, long long NP, const T *__restrict__ gz, T *gy)
{
    static_assert(KB == 16 || KB == 32, "KB lanes per chain");
    constexpr int CPW = 32 / KB;
    constexpr size_t TS = (size_t)KB * KB;
    __shared__ __align__(16) T vs[TWW_CHAINS * CPW][2][KB * HC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row = lane % KB;
    const int slot = warp * CPW + lane / KB;
    const int nch = (nrhs + HC - 1) / HC;
    const long long chain = (long long)blockIdx.x * TWW_CHAINS * CPW + slot;
    if (chain >= (long long)p * 2 * nch) return; // the whole chain
    const unsigned msk = tww_mask<KB>();
    const int part = (int)(chain / (2 * nch)), rem = (int)(chain - (long long)part * 2 * nch);
    const bool top = (rem & 1) == 0;
    const int h0 = (rem >> 1) * HC, nr = min(HC, nrhs - h0);
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const long long rb = (long long)blk_off[part] * KB;
    const int cnt = top ? M : N - 1 - M;
    T *yw = vs[slot][0], *tw = vs[slot][1];
    auto blk = [&](int i) { return top ? M - 1 - i : M + 1 + i; };
    auto fetch = [&](T (&d)[HC], int i) {
        const size_t rw = (size_t)rb + (size_t)blk(i) * KB + row;
#pragma unroll
        for (int h = 0; h < HC; h++) d[h] = h < nr ? gz[(size_t)(h0 + h) * NP + rw] : sc_zero<T>();
    };
    {
        T ym[HC]; // y_M
#pragma unroll
        for (int h = 0; h < HC; h++)
            ym[h] = h < nr ? gy[(size_t)(h0 + h) * NP + rb + (size_t)M * KB + row] : sc_zero<T>();
        vst<T, HC>(yw + row * HC, ym);
    }
    T zn[HC], gc[KB], ec[KB], gn[KB], en[KB];
    if (cnt > 0) {
        fetch(zn, 0);
        tww_row<T, KB>(gn, gG + tb + (size_t)blk(0) * TS, row);
        tww_row<T, KB>(en, gE + tb + (size_t)blk(0) * TS, row);
    }
    __syncwarp(msk);
    for (int i = 0; i < cnt; i++) {
        const int J = blk(i);
        T t[HC];
#pragma unroll
        for (int h = 0; h < HC; h++) t[h] = zn[h];
#pragma unroll
        for (int k = 0; k < KB; k++) {
            gc[k] = gn[k];
            ec[k] = en[k];
        }
        if (i + 1 < cnt) {
            fetch(zn, i + 1);
            tww_row<T, KB>(gn, gG + tb + (size_t)blk(i + 1) * TS, row);
            tww_row<T, KB>(en, gE + tb + (size_t)blk(i + 1) * TS, row);
        }
        tww_mv<T, KB, HC, true>(t, ec, yw); // z_J - A y_prev
        vst<T, HC>(tw + row * HC, t);
        __syncwarp(msk);
        T y[HC];
#pragma unroll
        for (int h = 0; h < HC; h++) y[h] = sc_zero<T>();
        tww_mv<T, KB, HC, false>(y, gc, tw); // G t
        __syncwarp(msk); // every lane of the chain has read y_prev and t
        vst<T, HC>(yw + row * HC, y);
#pragma unroll
        for (int h = 0; h < HC; h++)
            if (h < nr) gy[(size_t)(h0 + h) * NP + rb + (size_t)J * KB + row] = y[h];
        __syncwarp(msk);
    }
}

template <class T, int KB, int HC> int launch_tw_apply_w(spk_plan *P, const void *r, int nrhs, cudaStream_t st)
{
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t smem = tw_apply_smem<T, KB>();
    const long long chains = (long long)P->p * 2 * ((nrhs + HC - 1) / HC);
    const int per_cta = TWW_CHAINS * (32 / KB);
    const int grid = (int)((chains + per_cta - 1) / per_cta);
    k_tw_apply_fwd_w<T, KB, HC><<<grid, 32 * TWW_CHAINS, 0, st>>>(
        P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_L, (const T *)P->d_E,
        (const typename HighOf<T>::type *)r, P->n, nrhs, P->NP, (T *)P->d_z);
    SPK_CHECK_LAUNCH();
    const int hy = (nrhs + RC2 - 1) / RC2;
    k_tw_apply_mid<T, KB><<<dim3(P->p, hy), NT, smem, st>>>(P->d_blk_off, (const T *)P->d_L, (const T *)P->d_G, nrhs,
                                                            P->NP, (const T *)P->d_z, (T *)P->d_y);
    SPK_CHECK_LAUNCH();
    k_tw_apply_bwd_w<T, KB, HC><<<grid, 32 * TWW_CHAINS, 0, st>>>(P->d_blk_off, P->p, (const T *)P->d_G,
                                                                  (const T *)P->d_E, nrhs, P->NP, (const T *)P->d_z,
                                                                  (T *)P->d_y);
    SPK_CHECK_LAUNCH();
    P->launches += 3;
    return SPK_OK;
}

template <class T, int KB> int run_tw_apply(spk_plan *P, const void *r, int nrhs, cudaStream_t st)
{
    if constexpr (!TwistFits<T, KB>::ok) {
        return SPK_EBAND;
    } else {
        constexpr int NT = NTOf<KB>::value;
        constexpr size_t smem = tw_apply_smem<T, KB>();
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(k_tw_apply_fwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_tw_apply_mid<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_tw_apply_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                    cudaSuccess)
                return SPK_ECUDA;
            attr = true;
        }
        if constexpr (sizeof(T) == 4 && (KB == 16 || KB == 32)) { // KB lanes per chain
            if (nrhs == 1) return launch_tw_apply_w<T, KB, 1>(P, r, nrhs, st);
            if (nrhs <= 4) return launch_tw_apply_w<T, KB, 4>(P, r, nrhs, st);
            return launch_tw_apply_w<T, KB, 8>(P, r, nrhs, st);
        }
        const int hy = (nrhs + RC2 - 1) / RC2;
        k_tw_apply_fwd<T, KB><<<dim3(P->p, 2, hy), NT, smem, st>>>(
            P->d_part_start, P->d_blk_off, (const T *)P->d_L, (const T *)P->d_E,
            (const typename HighOf<T>::type *)r, P->n, nrhs, P->NP, (T *)P->d_z);
        SPK_CHECK_LAUNCH();
        k_tw_apply_mid<T, KB><<<dim3(P->p, hy), NT, smem, st>>>(P->d_blk_off, (const T *)P->d_L, (const T *)P->d_G,
                                                                nrhs, P->NP, (const T *)P->d_z, (T *)P->d_y);
        SPK_CHECK_LAUNCH();
        k_tw_apply_bwd<T, KB><<<dim3(P->p, 2, hy), NT, smem, st>>>(P->d_blk_off, (const T *)P->d_G,
                                                                   (const T *)P->d_E, nrhs, P->NP,
                                                                   (const T *)P->d_z, (T *)P->d_y);
        SPK_CHECK_LAUNCH();
        P->launches += 3;
        return SPK_OK;
    }
}

// g_i = (y_i bottom, y_{i+1} top), FP64 / complex128.
template <class T, int KB>
__global__ void k_ytips(const int *__restrict__ part_start, const int *__restrict__ blk_off, const T *__restrict__ gy,
                        long long NP, int nrhs, int n_iface, typename HighOf<T>::type *g)
{
    using H = typename HighOf<T>::type;
    const int i = blockIdx.x;
    const int mi = part_start[i + 1] - part_start[i];
    const long long NR = (long long)n_iface * 2 * KB;
    for (int q = threadIdx.x; q < 2 * KB * nrhs; q += blockDim.x) {
        const int h = q / (2 * KB), rr = q - h * 2 * KB;
        long long prow;
        if (rr < KB)
            prow = mi - KB + rr < 0 ? -1 : (long long)blk_off[i] * KB + (mi - KB + rr); // no bottom tip: see k_tips
        else
            prow = (long long)blk_off[i + 1] * KB + (rr - KB);
        g[h * NR + (long long)i * 2 * KB + rr] = prow < 0 ? sc_zero<H>() : cvt_fast<H, T>(gy[(size_t)h * NP + prow]);
    }
}

// x (+)= y - V_i t_{i+1} - W_i b_{i-1}; one CTA per (partition, block).
template <class T, int KB>
__global__ void __launch_bounds__(256)
    k_retrieve(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p, const int *__restrict__ blk_part,
               const T *__restrict__ gV, const T *__restrict__ gW, const T *__restrict__ gy,
               const T *__restrict__ u, long long NP, int n_iface, int n, int nrhs,
               typename HighOf<T>::type *x, int accumulate, const spk_sysref *__restrict__ sys,
               const int *__restrict__ part_sys)
{
    using H = typename HighOf<T>::type;
    constexpr size_t TS = (size_t)KB * KB;
    const int gb = blockIdx.x; // global block index
    const int part = blk_part[gb];
    const int J = gb - blk_off[part];
    int s = part_start[part];
    const int m = part_start[part + 1] - s;
    if (sys) { // batch group: write the partition's own system, local rows
        const spk_sysref &S = sys[part_sys[part]];
        x = (H *)S.x;
        n = S.n;
        s -= (int)S.row0;
    }
    const long long NR = (long long)n_iface * 2 * KB;
    const bool hasV = part < p - 1, hasW = part > 0;
    __shared__ T st[2 * KB * 8]; // interface unknowns in factor precision, converted once
    const int hchunk = 8;
    for (int hb = 0; hb < nrhs; hb += hchunk) {
        const int nr = min(hchunk, nrhs - hb);
        __syncthreads();
        for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
            const int c = q / nr, h = q - c * nr;
            st[c * hchunk + h] = hasV ? u[(hb + h) * NR + (long long)part * 2 * KB + KB + c] : sc_zero<T>();
            st[(KB + c) * hchunk + h] = hasW ? u[(hb + h) * NR + (long long)(part - 1) * 2 * KB + c] : sc_zero<T>();
        }
        __syncthreads();
        for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
            const int h = q / KB, lr = q - h * KB;
            const int lrow = J * KB + lr;
            if (lrow >= m) continue;
            T acc = gy[(size_t)(hb + h) * NP + (long long)gb * KB + lr];
            if (hasV)
                for (int c = 0; c < KB; c++)
                    acc = msub(acc, gV[(size_t)gb * TS + (size_t)c * KB + lr], st[c * hchunk + h]);
            if (hasW)
                for (int c = 0; c < KB; c++)
                    acc = msub(acc, gW[(size_t)gb * TS + (size_t)c * KB + lr], st[(KB + c) * hchunk + h]);
            H *xp = x + (size_t)(hb + h) * n + s + lrow;
            const H d = cvt_fast<H, T>(acc);
            *xp = accumulate ? *xp + d : d;
        }
    }
}

// ------------------------------------------------------------ small bands
// KB <= 8 (one-sided factors): KB lanes per (partition, column) chain.  Lane r owns row r of each
// block's vectors and tiles; z_{J-1} / y_{J+1} / t arrive by shuffles.  A ring
// entry holds the block's L (forward) or G and E (backward) tiles plus each
// lane's own right-hand-side or z element; z is kept in gy between the sweeps
// (each lane rereads only what it wrote).
template <class T, int KB> struct QuadApply {
    using H = typename HighOf<T>::type;
    static constexpr int TS = KB * KB;
    static constexpr int DEPTH = 4;
    static constexpr int VEC = 2 * TS * (int)sizeof(T); // byte offset of the lanes' elements
    static constexpr int STAGE = (VEC + KB * (int)sizeof(H) + 15) / 16 * 16;
    static constexpr int SLOT = DEPTH * STAGE + 16;
    static constexpr int CPC = chain_threads(SLOT);
    static constexpr int NT = CPC * KB;
    static constexpr size_t SMEM = (size_t)CPC * SLOT;
    static_assert(NT > 0 && NT <= 1024, "threads per CTA");
};

template <class T, int KB>
__global__ void __launch_bounds__(QuadApply<T, KB>::NT)
    k_quad_apply(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                 const T *__restrict__ gL, const T *__restrict__ gG, const T *__restrict__ gE,
                 const typename HighOf<T>::type *__restrict__ r, int n, int nrhs, long long NP, T *gy)
{
    using H = typename HighOf<T>::type;
    using C = QuadApply<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH;
    constexpr int CT = TS * (int)sizeof(T) / 16;
    extern __shared__ __align__(16) char smc[];
    const int ch = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int lr = threadIdx.x % KB;
    const int part = ch / nrhs, h = ch - part * nrhs;
    if (part >= p) return; // whole segments; no CTA barriers below
    const unsigned m = seg_mask<KB>();
    char *slot = smc + (threadIdx.x / KB) * C::SLOT;
    const int s = part_start[part], mrows = part_start[part + 1] - s;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    T *yh = gy + (size_t)h * NP + (size_t)blk_off[part] * KB;
    const H *rh = r + (size_t)h * n + s;

    // forward: z_J = r_J - L_J z_{J-1}
    auto issue_f = [&](int j) {
        if (j < N) {
            char *st = slot + (j % D) * C::STAGE;
            if (j > 0)
                for (int q = lr; q < CT; q += KB)
                    cp_async16(st + 16 * q, (const char *)(gL + tb + (size_t)j * TS) + 16 * q);
            if (j * KB + lr < mrows) cp_async_elem<(int)sizeof(H)>(st + C::VEC + lr * sizeof(H), rh + j * KB + lr);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int j = 0; j < D - 1; j++) issue_f(j);
    T z = sc_zero<T>();
    for (int J = 0; J < N; J++) {
        issue_f(J + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
        const char *st = slot + (J % D) * C::STAGE;
        T v = J * KB + lr < mrows ? sc_cvt<T, H>(*(const H *)(st + C::VEC + lr * sizeof(H))) : sc_zero<T>();
        if (J > 0) {
            const T *L = (const T *)st;
#pragma unroll
            for (int c = 0; c < KB; c++) v = msub(v, L[c * KB + lr], seg_shfl<KB>(m, z, c));
        }
        __syncwarp(m); // the ring entry may be refilled from here on
        z = v;
        yh[(size_t)J * KB + lr] = z;
    }
    cp_async_wait_all();
    __threadfence_block(); // the z stores above precede the copies below that read them back
    // backward: y_J = G_J (z_J - E_J y_{J+1}); step i handles block N-1-i
    auto issue_b = [&](int i) {
        if (i < N) {
            const int J = N - 1 - i;
            char *st = slot + (i % D) * C::STAGE;
            for (int q = lr; q < CT; q += KB) {
                cp_async16(st + 16 * q, (const char *)(gG + tb + (size_t)J * TS) + 16 * q);
                cp_async16(st + TS * sizeof(T) + 16 * q, (const char *)(gE + tb + (size_t)J * TS) + 16 * q);
            }
            cp_async_elem<(int)sizeof(T)>(st + C::VEC + lr * sizeof(T), yh + (size_t)J * KB + lr); // own z element
        }
        cp_async_commit();
    };
#pragma unroll
    for (int i = 0; i < D - 1; i++) issue_b(i);
    T y = sc_zero<T>();
    for (int i = 0; i < N; i++) {
        const int J = N - 1 - i;
        issue_b(i + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
        const char *st = slot + (i % D) * C::STAGE;
        const T *G = (const T *)st, *E = (const T *)(st + TS * sizeof(T));
        T t = *(const T *)(st + C::VEC + lr * sizeof(T));
        if (J < N - 1)
#pragma unroll
            for (int c = 0; c < KB; c++) t = msub(t, E[c * KB + lr], seg_shfl<KB>(m, y, c));
        T acc = sc_zero<T>();
#pragma unroll
        for (int c = 0; c < KB; c++) acc = madd(acc, G[c * KB + lr], seg_shfl<KB>(m, t, c));
        __syncwarp(m);
        y = acc;
        yh[(size_t)J * KB + lr] = y;
    }
    cp_async_wait_all();
}

// interface unknowns u (FP64 / complex128) -> factor precision
// Two-sided partitions, KB <= 4 (the factors' layout of spike_twist.cu):
// chains per (partition, column) and half.  k_qtw_apply_fwd runs the top
// half's z_J = r_J - L_J z_{J-1} (J < M) and the bottom half's
// w_J = r_J - U_J w_{J+1} (J >= M) into y; k_qtw_apply_mid forms
// y_M = G_M (w_M - L_M z_{M-1}); k_qtw_apply_bwd runs y_J = G_J (z_J -
// A(J,J+1) y_{J+1}) upwards and y_J = H_J (w_J - A(J,J-1) y_{J-1}) downwards.
// The lane sweeps' ring: a stage carries S consecutive steps' tiles and
// vector elements, so a chain waits and synchronises once per S steps.
template <class T, int KB> struct QTwApply {
    using H = typename HighOf<T>::type;
    static constexpr int TS = KB * KB;
    static constexpr int S = 4;                                  // steps per stage
    static constexpr int DEPTH = 3;                              // stages in flight
    static constexpr int VEC = 2 * TS * (int)sizeof(T);          // byte offset of a step's vector elements
    static constexpr int STEP = (VEC + KB * (int)sizeof(H) + 15) / 16 * 16;
    static constexpr int STAGE = S * STEP;
    static constexpr int SLOT = DEPTH * STAGE + 16;
    static constexpr int CPC = chain_threads(SLOT);
    static constexpr int NT = CPC * KB;
    static constexpr size_t SMEM = (size_t)CPC * SLOT;
};

template <class T, int KB>
__global__ void __launch_bounds__(QTwApply<T, KB>::NT)
    k_qtw_apply_fwd(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                    const T *__restrict__ gL, const T *__restrict__ gE,
                    const typename HighOf<T>::type *__restrict__ r, int n, int nrhs, long long NP, T *gy)
{
    using H = typename HighOf<T>::type;
    using C = QTwApply<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH, S = C::S;
    constexpr int CT = TS * (int)sizeof(T) / 16;
    extern __shared__ __align__(16) char smc[];
    const int ch = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int lr = threadIdx.x % KB;
    const int pc = ch >> 1;
    const bool bottom = ch & 1;
    const int part = pc / nrhs, h = pc - part * nrhs;
    if (part >= p) return; // whole segments; no CTA barriers below
    const unsigned m = seg_mask<KB>();
    char *slot = smc + (threadIdx.x / KB) * C::SLOT;
    const int s = part_start[part], mrows = part_start[part + 1] - s;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    T *yh = gy + (size_t)h * NP + (size_t)blk_off[part] * KB;
    const H *rh = r + (size_t)h * n + s;
    const int cnt = bottom ? N - M : M;
    auto blk = [&](int i) { return bottom ? N - 1 - i : i; };
    auto issue = [&](int g) { // stage g: steps g*S .. g*S+S-1
#pragma unroll
        for (int q = 0; q < S; q++) {
            const int i = g * S + q;
            if (i < cnt) {
                const int J = blk(i);
                char *st = slot + (g % D) * C::STAGE + q * C::STEP;
                if (i > 0) { // the coupling tile: L_J above M, U_J below (U_M in gE)
                    const T *cpl = (bottom && J == M ? gE : gL) + tb + (size_t)J * TS;
                    for (int k = lr; k < CT; k += KB) cp_async16(st + 16 * k, (const char *)cpl + 16 * k);
                }
                if (J * KB + lr < mrows)
                    cp_async_elem<(int)sizeof(H)>(st + C::VEC + lr * sizeof(H), rh + J * KB + lr);
            }
        }
        cp_async_commit();
    };
    const int ng = (cnt + S - 1) / S;
#pragma unroll
    for (int g = 0; g < D - 1; g++) issue(g);
    T z = sc_zero<T>();
    for (int g = 0; g < ng; g++) {
        issue(g + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
#pragma unroll
        for (int q = 0; q < S; q++) {
            const int i = g * S + q;
            if (i < cnt) {
                const int J = blk(i);
                const char *st = slot + (g % D) * C::STAGE + q * C::STEP;
                T v = J * KB + lr < mrows ? sc_cvt<T, H>(*(const H *)(st + C::VEC + lr * sizeof(H))) : sc_zero<T>();
                if (i > 0) {
                    const T *L = (const T *)st; // column-major
#pragma unroll
                    for (int c = 0; c < KB; c++) v = msub(v, L[c * KB + lr], seg_shfl<KB>(m, z, c));
                }
                z = v;
                yh[(size_t)J * KB + lr] = z;
            }
        }
        __syncwarp(m); // the stage may be refilled from here on
    }
    cp_async_wait_all();
}

template <class T, int KB>
__global__ void k_qtw_apply_mid(const int *__restrict__ blk_off, int p, const T *__restrict__ gL,
                                const T *__restrict__ gG, int nrhs, long long NP, T *gy)
{
    constexpr int TS = KB * KB;
    const int ch = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int lr = threadIdx.x % KB;
    const int part = ch / nrhs, h = ch - part * nrhs;
    if (part >= p) return; // whole segments
    const unsigned m = seg_mask<KB>();
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    T *yh = gy + (size_t)h * NP + (size_t)blk_off[part] * KB;
    const T zp = yh[(size_t)(M - 1) * KB + lr];
    T v = yh[(size_t)M * KB + lr]; // w_M
#pragma unroll
    for (int c = 0; c < KB; c++) v = msub(v, gL[tb + (size_t)M * TS + c * KB + lr], seg_shfl<KB>(m, zp, c));
    T y = sc_zero<T>();
#pragma unroll
    for (int c = 0; c < KB; c++) y = madd(y, gG[tb + (size_t)M * TS + c * KB + lr], seg_shfl<KB>(m, v, c));
    yh[(size_t)M * KB + lr] = y;
}

template <class T, int KB>
__global__ void __launch_bounds__(QTwApply<T, KB>::NT)
    k_qtw_apply_bwd(const int *__restrict__ blk_off, int p, const T *__restrict__ gG, const T *__restrict__ gE,
                    int nrhs, long long NP, T *gy)
{
    using C = QTwApply<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH, S = C::S;
    constexpr int CT = TS * (int)sizeof(T) / 16;
    extern __shared__ __align__(16) char smc[];
    const int ch = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int lr = threadIdx.x % KB;
    const int pc = ch >> 1;
    const bool bottom = ch & 1;
    const int part = pc / nrhs, h = pc - part * nrhs;
    if (part >= p) return; // whole segments; no CTA barriers below
    const unsigned m = seg_mask<KB>();
    char *slot = smc + (threadIdx.x / KB) * C::SLOT;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    T *yh = gy + (size_t)h * NP + (size_t)blk_off[part] * KB;
    const int cnt = bottom ? N - 1 - M : M;
    auto blk = [&](int i) { return bottom ? M + 1 + i : M - 1 - i; };
    auto issue = [&](int g) {
#pragma unroll
        for (int q = 0; q < S; q++) {
            const int i = g * S + q;
            if (i < cnt) {
                const int J = blk(i);
                char *st = slot + (g % D) * C::STAGE + q * C::STEP;
                for (int k = lr; k < CT; k += KB) {
                    cp_async16(st + 16 * k, (const char *)(gG + tb + (size_t)J * TS) + 16 * k);
                    cp_async16(st + TS * sizeof(T) + 16 * k, (const char *)(gE + tb + (size_t)J * TS) + 16 * k);
                }
                // the forward sweep's own z_J / w_J: y_J is written only when the chain gets there
                cp_async_elem<(int)sizeof(T)>(st + C::VEC + lr * sizeof(T), yh + (size_t)J * KB + lr);
            }
        }
        cp_async_commit();
    };
    const int ng = (cnt + S - 1) / S;
#pragma unroll
    for (int g = 0; g < D - 1; g++) issue(g);
    T y = yh[(size_t)M * KB + lr]; // y_M
    for (int g = 0; g < ng; g++) {
        issue(g + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
#pragma unroll
        for (int q = 0; q < S; q++) {
            const int i = g * S + q;
            if (i < cnt) {
                const char *st = slot + (g % D) * C::STAGE + q * C::STEP;
                const T *G = (const T *)st, *E = (const T *)(st + TS * sizeof(T));
                T t = *(const T *)(st + C::VEC + lr * sizeof(T));
#pragma unroll
                for (int c = 0; c < KB; c++) t = msub(t, E[c * KB + lr], seg_shfl<KB>(m, y, c));
                T acc = sc_zero<T>();
#pragma unroll
                for (int c = 0; c < KB; c++) acc = madd(acc, G[c * KB + lr], seg_shfl<KB>(m, t, c));
                y = acc;
                yh[(size_t)blk(i) * KB + lr] = y;
            }
        }
        __syncwarp(m);
    }
    cp_async_wait_all();
}

template <class T>
__global__ void k_u_narrow(const typename HighOf<T>::type *__restrict__ u, T *ut, long long count)
{
    using H = typename HighOf<T>::type;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < count;
         q += (long long)gridDim.x * blockDim.x)
        ut[q] = cvt_fast<T, H>(u[q]);
}

// x (+)= y - V_i t_{i+1} - W_i b_{i-1} for tiles of 8 to 32 rows: one thread per
// (padded row, pass of eight right-hand-side columns), consecutive threads on
// consecutive rows (a CTA per row block would leave most of its threads
// idle).  Each V and W entry a row needs is loaded once per pass and applied
// to all of the pass's columns, so at up to eight columns the spikes cross
// HBM once per call; wider right-hand sides keep one thread per pass, so a
// small system with many columns still fills the GPU.
constexpr int RET_HC = 8; // right-hand-side columns per pass of k_retrieve_rows

template <class T, int KB>
__global__ void __launch_bounds__(256)
    k_retrieve_rows(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                    const int *__restrict__ blk_part, const T *__restrict__ gV, const T *__restrict__ gW,
                    const T *__restrict__ gy, const T *__restrict__ ut, long long NP, int n_iface, int n, int nrhs,
                    typename HighOf<T>::type *x, int accumulate, const spk_sysref *__restrict__ sys,
                    const int *__restrict__ part_sys)
{
    using H = typename HighOf<T>::type;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int HC = RET_HC;
    const long long NR = (long long)n_iface * 2 * KB;
    const long long tot = NP * ((nrhs + HC - 1) / HC);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < tot;
         q += (long long)gridDim.x * blockDim.x) {
        const int h0 = (int)(q / NP) * HC;
        const long long pr = q - (long long)(h0 / HC) * NP;
        const int gb = (int)(pr / KB), lr = (int)(pr - (long long)gb * KB);
        const int part = blk_part[gb];
        const int lrow = (gb - blk_off[part]) * KB + lr;
        int s = part_start[part];
        if (lrow >= part_start[part + 1] - s) continue; // identity padding row
        H *xb = x;
        int ld = n;
        if (sys) {
            const spk_sysref &S = sys[part_sys[part]];
            xb = (H *)S.x;
            ld = S.n;
            s -= (int)S.row0;
        }
        const bool hasV = part < p - 1, hasW = part > 0;
        const int nh = min(HC, nrhs - h0);
        T acc[HC];
#pragma unroll
        for (int hh = 0; hh < HC; hh++) acc[hh] = hh < nh ? gy[(size_t)(h0 + hh) * NP + pr] : sc_zero<T>();
        if (hasV) {
            const T *t = ut + (size_t)h0 * NR + (size_t)part * 2 * KB + KB;
#pragma unroll 4
            for (int c = 0; c < KB; c++) {
                const T vc = gV[(size_t)gb * TS + (size_t)c * KB + lr];
#pragma unroll
                for (int hh = 0; hh < HC; hh++)
                    if (hh < nh) acc[hh] = msub(acc[hh], vc, t[(size_t)hh * NR + c]);
            }
        }
        if (hasW) {
            const T *bw = ut + (size_t)h0 * NR + (size_t)(part - 1) * 2 * KB;
#pragma unroll 4
            for (int c = 0; c < KB; c++) {
                const T wc = gW[(size_t)gb * TS + (size_t)c * KB + lr];
#pragma unroll
                for (int hh = 0; hh < HC; hh++)
                    if (hh < nh) acc[hh] = msub(acc[hh], wc, bw[(size_t)hh * NR + c]);
            }
        }
#pragma unroll
        for (int hh = 0; hh < HC; hh++)
            if (hh < nh) {
                H *xp = xb + (size_t)(h0 + hh) * ld + s + lrow;
                const H d = cvt_fast<H, T>(acc[hh]);
                *xp = accumulate ? *xp + d : d;
            }
    }
}

// The same for tiles of up to 4 rows: one thread per (padded row, column),
// the column varying fastest.  The independent (row, column) items keep more
// arithmetic in flight than a loop over the columns, and a row's columns sit
// on neighbouring lanes, so they share each load of the row's spike entries:
// the spikes cross from DRAM once, not once per column (at 4-row complex
// tiles and 4 million rows they are 256 MB, twice the L2).
template <class T, int KB>
__global__ void __launch_bounds__(256)
    k_retrieve_rc(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                    const int *__restrict__ blk_part, const T *__restrict__ gV, const T *__restrict__ gW,
                    const T *__restrict__ gy, const T *__restrict__ ut, long long NP, int n_iface, int n, int nrhs,
                    typename HighOf<T>::type *x, int accumulate, const spk_sysref *__restrict__ sys,
                    const int *__restrict__ part_sys)
{
    using H = typename HighOf<T>::type;
    constexpr size_t TS = (size_t)KB * KB;
    const long long NR = (long long)n_iface * 2 * KB;
    const long long tot = NP * nrhs;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < tot;
         q += (long long)gridDim.x * blockDim.x) {
        const long long pr = q / nrhs;
        const int h = (int)(q - pr * nrhs);
        const int gb = (int)(pr / KB), lr = (int)(pr - (long long)gb * KB);
        const int part = blk_part[gb];
        const int lrow = (gb - blk_off[part]) * KB + lr;
        int s = part_start[part];
        if (lrow >= part_start[part + 1] - s) continue; // identity padding row
        H *xb = x;
        int ld = n;
        if (sys) {
            const spk_sysref &S = sys[part_sys[part]];
            xb = (H *)S.x;
            ld = S.n;
            s -= (int)S.row0;
        }
        T acc = gy[(size_t)h * NP + pr];
        if (part < p - 1) {
            const T *t = ut + (size_t)h * NR + (size_t)part * 2 * KB + KB;
#pragma unroll
            for (int c = 0; c < KB; c++) acc = msub(acc, gV[(size_t)gb * TS + (size_t)c * KB + lr], t[c]);
        }
        if (part > 0) {
            const T *bw = ut + (size_t)h * NR + (size_t)(part - 1) * 2 * KB;
#pragma unroll
            for (int c = 0; c < KB; c++) acc = msub(acc, gW[(size_t)gb * TS + (size_t)c * KB + lr], bw[c]);
        }
        H *xp = xb + (size_t)h * ld + s + lrow;
        const H d = cvt_fast<H, T>(acc);
        *xp = accumulate ? *xp + d : d;
    }
}

// the lane kernel's ring of 8-row tiles fits shared memory (not for complex128)
template <class T> constexpr bool quad_apply_8_fits() { return QuadApply<T, 8>::SMEM <= 227 * 1024; }

template <class T, int KB> int run_apply_1(spk_plan *P, const void *r, int nrhs, cudaStream_t st)
{
    constexpr int NT = NTOf<KB>::value;
    const size_t smem = 16 + sizeof(T) * ((KB >= 128 ? 2 : 4) * KB * TileLD<T, KB>::value + 3 * KB * RCS);
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_apply<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return SPK_ECUDA;
        attr = true;
    }
    // KB lanes per (partition, column) chain up to 8-row tiles (where the ring
    // of 8-row tiles fits shared memory): a step is KB shuffles and
    // multiply-adds per lane, where the CTA kernel pays a barrier per step
    if constexpr (KB <= 4 || (KB == 8 && quad_apply_8_fits<T>())) {
        using CA = QuadApply<T, KB>;
        static bool cattr = false;
        if (!cattr) {
            if (cudaFuncSetAttribute(k_quad_apply<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)CA::SMEM) != cudaSuccess)
                return SPK_ECUDA;
            cattr = true;
        }
        const long long chains = (long long)P->p * nrhs;
        const int cpc = chains_per_cta(chains, CA::CPC);
        k_quad_apply<T, KB><<<(int)((chains + cpc - 1) / cpc), cpc * KB, (size_t)cpc * CA::SLOT, st>>>(
            P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_L, (const T *)P->d_G, (const T *)P->d_E,
            (const typename HighOf<T>::type *)r, P->n, nrhs, P->NP, (T *)P->d_y);
    } else {
        dim3 grid(P->p, (nrhs + RC - 1) / RC);
        k_apply<T, KB><<<grid, NT, smem, st>>>(P->d_part_start, P->d_blk_off, (const T *)P->d_L, (const T *)P->d_G,
                                               (const T *)P->d_E, (const typename HighOf<T>::type *)r, P->n, nrhs,
                                               P->NP, (T *)P->d_z, (T *)P->d_y);
    }
    SPK_CHECK_LAUNCH();
    P->launches++;
    return SPK_OK;
}

template <class T, int KB> int run_qtw_apply(spk_plan *P, const void *r, int nrhs, cudaStream_t st)
{
    using CA = QTwApply<T, KB>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_qtw_apply_fwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)CA::SMEM) != cudaSuccess ||
            cudaFuncSetAttribute(k_qtw_apply_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)CA::SMEM) != cudaSuccess)
            return SPK_ECUDA;
        attr = true;
    }
    const long long chains = 2LL * P->p * nrhs;
    const int cpc = chains_per_cta(chains, CA::CPC);
    k_qtw_apply_fwd<T, KB><<<(int)((chains + cpc - 1) / cpc), cpc * KB, (size_t)cpc * CA::SLOT, st>>>(
        P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_L, (const T *)P->d_E,
        (const typename HighOf<T>::type *)r, P->n, nrhs, P->NP, (T *)P->d_y);
    SPK_CHECK_LAUNCH();
    const long long mch = (long long)P->p * nrhs;
    k_qtw_apply_mid<T, KB><<<(int)((mch + 31) / 32), 32 * KB, 0, st>>>(P->d_blk_off, P->p, (const T *)P->d_L,
                                                                       (const T *)P->d_G, nrhs, P->NP, (T *)P->d_y);
    SPK_CHECK_LAUNCH();
    k_qtw_apply_bwd<T, KB><<<(int)((chains + cpc - 1) / cpc), cpc * KB, (size_t)cpc * CA::SLOT, st>>>(
        P->d_blk_off, P->p, (const T *)P->d_G, (const T *)P->d_E, nrhs, P->NP, (T *)P->d_y);
    SPK_CHECK_LAUNCH();
    P->launches += 3;
    return SPK_OK;
}

template <class T, int KB> int run_apply(spk_plan *P, const void *r, int nrhs, cudaStream_t st)
{
    int rc;
    if constexpr (KB <= 4)
        rc = P->twist ? run_qtw_apply<T, KB>(P, r, nrhs, st) : run_apply_1<T, KB>(P, r, nrhs, st);
    else
        rc = P->twist ? run_tw_apply<T, KB>(P, r, nrhs, st) : run_apply_1<T, KB>(P, r, nrhs, st);
    if (rc != SPK_OK) return rc;
    if (P->n_iface > 0) {
        k_ytips<T, KB><<<P->n_iface, 128, 0, st>>>(P->d_part_start, P->d_blk_off, (const T *)P->d_y, P->NP, nrhs,
                                                   P->n_iface, (typename HighOf<T>::type *)P->d_g);
        SPK_CHECK_LAUNCH();
        P->launches++;
    }
    return SPK_OK;
}

template <class T, int KB> int run_retrieve(spk_plan *P, void *x, int nrhs, int accumulate, cudaStream_t st)
{
    using H = typename HighOf<T>::type;
    // the interface unknowns, narrowed once into the (now free) reduced-RHS work array
    T *ut = (T *)P->d_crg;
    const long long cnt = (long long)(P->n_iface > 0 ? P->n_iface : 1) * 2 * KB * nrhs;
    if (P->n_iface > 0) {
        k_u_narrow<T><<<(int)std::min<long long>((cnt + 255) / 256, 4096), 256, 0, st>>>((const H *)P->d_u, ut, cnt);
        SPK_CHECK_LAUNCH();
        P->launches++;
    }
    if constexpr (KB <= 32) {
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int cap = (sms > 0 ? sms : 152) * 8;
        if constexpr (KB <= 4) {
            const long long tot = P->NP * nrhs;
            const int grid = (int)std::min<long long>((tot + 255) / 256, (long long)cap);
            k_retrieve_rc<T, KB><<<grid, 256, 0, st>>>(P->d_part_start, P->d_blk_off, P->p, P->d_blk_part,
                                                       (const T *)P->d_V, (const T *)P->d_W, (const T *)P->d_y, ut,
                                                       P->NP, P->n_iface, P->n, nrhs, (H *)x, accumulate, P->d_sys,
                                                       P->d_part_sys);
        } else {
            const long long tot = P->NP * ((nrhs + RET_HC - 1) / RET_HC);
            const int grid = (int)std::min<long long>((tot + 255) / 256, (long long)cap);
            k_retrieve_rows<T, KB><<<grid, 256, 0, st>>>(P->d_part_start, P->d_blk_off, P->p, P->d_blk_part,
                                                         (const T *)P->d_V, (const T *)P->d_W, (const T *)P->d_y, ut,
                                                         P->NP, P->n_iface, P->n, nrhs, (H *)x, accumulate, P->d_sys,
                                                         P->d_part_sys);
        }
    } else {
        k_retrieve<T, KB><<<P->total_blocks, 256, 0, st>>>(P->d_part_start, P->d_blk_off, P->p, P->d_blk_part,
                                                           (const T *)P->d_V, (const T *)P->d_W, (const T *)P->d_y,
                                                           ut, P->NP, P->n_iface, P->n, nrhs, (H *)x, accumulate,
                                                           P->d_sys, P->d_part_sys);
    }
    SPK_CHECK_LAUNCH();
    P->launches++;
    return SPK_OK;
}

#define SPK_KB_SWITCH(FN, T, ...)                                                                               \
    switch (P->KB) {                                                                                            \
    case 2: return FN<T, 2>(__VA_ARGS__);                                                                       \
    case 4: return FN<T, 4>(__VA_ARGS__);                                                                       \
    case 8: return FN<T, 8>(__VA_ARGS__);                                                                       \
    case 16: return FN<T, 16>(__VA_ARGS__);                                                                     \
    case 32: return FN<T, 32>(__VA_ARGS__);                                                                     \
    case 64:                                                                                                    \
        if constexpr (sizeof(T) <= 8) return FN<T, 64>(__VA_ARGS__);                                            \
        else return SPK_EBAND;                                                                                  \
    case 128:                                                                                                   \
        if constexpr (std::is_same<T, float>::value) return FN<T, 128>(__VA_ARGS__);                            \
        else return SPK_EBAND;                                                                                  \
    default: return SPK_EBAND;                                                                                  \
    }

template <class T> int disp_apply(spk_plan *P, const void *r, int nrhs, cudaStream_t st)
{
    SPK_KB_SWITCH(run_apply, T, P, r, nrhs, st)
}
template <class T> int disp_retrieve(spk_plan *P, void *x, int nrhs, int acc, cudaStream_t st)
{
    SPK_KB_SWITCH(run_retrieve, T, P, x, nrhs, acc, st)
}

} // namespace

extern "C" int spk_apply(spk_plan *P, const void *d_r, int nrhs, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (P->is_complex)
        return P->mode == SPK_MIXED ? disp_apply<cfloat>(P, d_r, nrhs, st) : disp_apply<cdouble>(P, d_r, nrhs, st);
    return P->mode == SPK_MIXED ? disp_apply<float>(P, d_r, nrhs, st) : disp_apply<double>(P, d_r, nrhs, st);
}

extern "C" int spk_retrieve(spk_plan *P, void *d_x, int nrhs, int accumulate, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (P->is_complex)
        return P->mode == SPK_MIXED ? disp_retrieve<cfloat>(P, d_x, nrhs, accumulate, st)
                                    : disp_retrieve<cdouble>(P, d_x, nrhs, accumulate, st);
    return P->mode == SPK_MIXED ? disp_retrieve<float>(P, d_x, nrhs, accumulate, st)
                                : disp_retrieve<double>(P, d_x, nrhs, accumulate, st);
}
