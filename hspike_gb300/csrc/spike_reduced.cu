// spike_reduced.cu -- the reduced system of the SPIKE solve on sm_103a.
//
// The reference assembles R as a CSR matrix (matrix_CreateEmptyReducedSystem
// and matrix_AddTipToReducedMatrix, OpenMP/spike_matrix.c:657-740,1414-1495)
// and solves it with MKL PARDISO on the host (directSolver_Host_Solve,
// OpenMP/spike_algebra.c:263-420).  Here R stays on the device in its natural
// block form.  With one 2KB-vector of unknowns per interface i,
// u_i = (b_i, t_{i+1}), R is block tridiagonal:
//
//     D_i = [[I, P_i], [Q_i, I]]     P_i = V_i bottom tip, Q_i = W_{i+1} top tip
//     A_i = [[X_i, 0], [0, 0]]       X_i = W_i bottom tip       (couples u_{i-1})
//     C_i = [[0, 0], [0, Y_i]]       Y_i = V_{i+1} top tip      (couples u_{i+1})
//
// Block cyclic reduction keeps that quadrant structure at every level (the
// products A M C, C M A, A M A, C M C each fill a single KB x KB quadrant), so
// a level costs ~13 KB^3 multiply-adds per eliminated pair instead of the
// dense (2KB)^3 form.  The factorization runs in the factor precision
// (FP32/complex64 in mixed mode, FP64 in plain mode); the solve wraps it in
// FP64 refinement on R itself, u += CR^{-1}(g - R u), so the reduced solution
// is FP64-accurate in both modes.
#include "spike_common.cuh"

#include <type_traits>

namespace {

template <class T, int KB> struct RedSmem {
    using TL = Tile<T, KB, NTOf<KB>::value>;
    static constexpr size_t bytes = 3 * sizeof(T) * TL::ELEMS + sizeof(T) * TL::INV_BUF + 64;
    static constexpr size_t solve = sizeof(T) * KB * TileLD<T, KB>::value + 64; // one tile (k_cr_fwd / k_cr_bwd)
};

template <class T, int KB> __device__ void ld(T *s, const T *g)
{
    copy_tile_g2s<T, KB, NTOf<KB>::value>(s, g);
}
template <class T, int KB, class Reg> __device__ void set_identity(const Tile<T, KB, NTOf<KB>::value> &t, Reg &a)
{
#pragma unroll
    for (int i = 0; i < t.TR; i++)
#pragma unroll
        for (int j = 0; j < t.TC; j++) a[i][j] = (t.row(i) == t.col(j)) ? sc_one<T>() : sc_zero<T>();
}

// level-0 blocks: FP64 -> factor precision
template <class T>
__global__ void k_red_cvt(const typename HighOf<T>::type *__restrict__ src, T *dst, long long count)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < count; q += (long long)gridDim.x * blockDim.x)
        dst[q] = cvt_fast<T, typename HighOf<T>::type>(src[q]);
}

// Odd blocks j of a level (or the single top block): M = D_j^{-1} by quadrants
//   S = I - Q P, M11 = S^{-1}, M10 = -M11 Q, M01 = -P M11, M00 = I - P M10.
// Three shared tiles: P, Q (overwritten by M10 once M10 exists) and M11.
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_cr_odd(const T *__restrict__ Pl, const T *__restrict__ Ql, int first, int stride, T *M, unsigned *err)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    const int j = first + blockIdx.x * stride;
    T *Mj = M + (size_t)blockIdx.x * 4 * TS;
    extern __shared__ char smraw[];
    T *sP = (T *)smem_align(smraw), *sQ = sP + TL::ELEMS, *sH = sQ + TL::ELEMS;
    T *buf = sH + TL::ELEMS;
    TL t(threadIdx.x);
    typename TL::Reg a;
    ld<T, KB>(sP, Pl + (size_t)j * TS);
    ld<T, KB>(sQ, Ql + (size_t)j * TS);
    __syncthreads();
    set_identity<T, KB>(t, a);
    t.mms(a, sQ, sP);
    const bool ok = t.inverse(a, buf);
    if (!ok && threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
    t.rstore(sH, a);
    t.gstore(Mj + 3 * TS, a);
    __syncthreads();
    t.rzero(a);
    t.mms(a, sH, sQ); // M10
    t.gstore(Mj + 2 * TS, a);
    __syncthreads(); // every read of Q is done
    t.rstore(sQ, a);
    t.rzero(a);
    t.mms(a, sP, sH); // M01
    t.gstore(Mj + 1 * TS, a);
    __syncthreads();
    set_identity<T, KB>(t, a);
    t.mms(a, sP, sQ); // M00 = I - P M10
    t.gstore(Mj, a);
}

// acc += sign * L (M R); L, M, R global tiles; uses sA, sB, sC
template <class T, int KB>
__device__ __forceinline__ void chain3(const Tile<T, KB, NTOf<KB>::value> &t, typename Tile<T, KB, NTOf<KB>::value>::Reg &acc,
                       const T *L, const T *Mg, const T *R, T *sA, T *sB, T *sC, bool negate)
{
    typename Tile<T, KB, NTOf<KB>::value>::Reg tmp;
    __syncthreads();
    ld<T, KB>(sA, Mg);
    ld<T, KB>(sB, R);
    __syncthreads();
    t.rzero(tmp);
    t.mma(tmp, sA, sB);
    t.rstore(sC, tmp);
    __syncthreads();
    ld<T, KB>(sA, L);
    __syncthreads();
    if (negate)
        t.mms(acc, sA, sC);
    else
        t.mma(acc, sA, sC);
}

// Even blocks i of level l produce block i/2 of level l+1:
//   P' = P_i - X_i M01_{i-1} Y_{i-1}    Q' = Q_i - Y_i M10_{i+1} X_{i+1}
//   X' = -X_i M00_{i-1} X_{i-1}         Y' = -Y_i M11_{i+1} Y_{i+1}
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_cr_even(const T *__restrict__ Pl, const T *__restrict__ Ql, const T *__restrict__ Xl, const T *__restrict__ Yl,
              const T *__restrict__ Ml, int cnt, T *Pn, T *Qn, T *Xn, T *Yn)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    const int i = 2 * blockIdx.x, a_out = blockIdx.x;
    extern __shared__ char smraw[];
    T *sA = (T *)smem_align(smraw), *sB = sA + TL::ELEMS, *sC = sB + TL::ELEMS;
    TL t(threadIdx.x);
    typename TL::Reg acc;
    const bool left = i - 1 >= 0, right = i + 1 < cnt;
    const T *Ml_left = left ? Ml + (size_t)((i - 2) / 2) * 4 * TS : nullptr;  // odd block i-1
    const T *Ml_right = right ? Ml + (size_t)(i / 2) * 4 * TS : nullptr;      // odd block i+1
    // the four results are independent: one CTA each (blockIdx.y), so a level
    // of few blocks still spreads over the SMs
    switch (blockIdx.y) {
    case 0: // P'
        ld<T, KB>(sA, Pl + (size_t)i * TS);
        __syncthreads();
        t.rload(acc, sA);
        if (left)
            chain3<T, KB>(t, acc, Xl + (size_t)i * TS, Ml_left + 1 * TS, Yl + (size_t)(i - 1) * TS, sA, sB, sC, true);
        t.gstore(Pn + (size_t)a_out * TS, acc);
        break;
    case 1: // Q'
        ld<T, KB>(sA, Ql + (size_t)i * TS);
        __syncthreads();
        t.rload(acc, sA);
        if (right)
            chain3<T, KB>(t, acc, Yl + (size_t)i * TS, Ml_right + 2 * TS, Xl + (size_t)(i + 1) * TS, sA, sB, sC, true);
        t.gstore(Qn + (size_t)a_out * TS, acc);
        break;
    case 2: // X'
        t.rzero(acc);
        if (left)
            chain3<T, KB>(t, acc, Xl + (size_t)i * TS, Ml_left + 0 * TS, Xl + (size_t)(i - 1) * TS, sA, sB, sC, true);
        t.gstore(Xn + (size_t)a_out * TS, acc);
        break;
    default: // Y'
        t.rzero(acc);
        if (right)
            chain3<T, KB>(t, acc, Yl + (size_t)i * TS, Ml_right + 3 * TS, Yl + (size_t)(i + 1) * TS, sA, sB, sC, true);
        t.gstore(Yn + (size_t)a_out * TS, acc);
    }
}

// ---------------------------------------------------------------- tensor-core products
// The reduced system's 2KB x 2KB block products for KB >= 64 (FP32 factors)
// run on the tensor cores: warp-level mma.sync m16n8k8 with TF32 operands,
// each FP32 operand split into a TF32 high part and a TF32 remainder, and
// the three significant partial products (lo*hi, hi*lo, hi*hi) accumulated
// in FP32, which keeps FP32 accuracy.  Warp w of the CTA (KB*KB/512 warps:
// the Tile kernels' own thread count) owns the 32 x 16 output block at rows
// 32 (w / (KB/16)), columns 16 (w % (KB/16)); operands are shared tiles in
// the Tile layout (row-major, row stride KB + 4).
__device__ __forceinline__ void tf32_split(float x, uint32_t &hi, uint32_t &lo)
{
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - __uint_as_float(h)));
    hi = h;
    lo = l;
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
using TcAcc = float[2][2][4];
__device__ __forceinline__ void tc_zero(TcAcc &acc)
{
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;
}
// acc += A B (A, B: KB x KB shared tiles, row-major, row stride KB + 4)
template <int KB> __device__ __forceinline__ void tc_mm(TcAcc &acc, const float *A, const float *B)
{
    constexpr int LD = TileLD<float, KB>::value;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = (warp / (KB / 16)) * 32, c0 = (warp % (KB / 16)) * 16;
#pragma unroll 2
    for (int k0 = 0; k0 < KB; k0 += 8) {
        uint32_t ah[2][4], al[2][4], bh[2][2], bl[2][2];
#pragma unroll
        for (int i = 0; i < 2; i++) { // A fragment: (g, t), (g + 8, t), (g, t + 4), (g + 8, t + 4)
            const float *Ar = A + (r0 + i * 16 + g) * LD + k0 + t;
            tf32_split(Ar[0], ah[i][0], al[i][0]);
            tf32_split(Ar[8 * LD], ah[i][1], al[i][1]);
            tf32_split(Ar[4], ah[i][2], al[i][2]);
            tf32_split(Ar[8 * LD + 4], ah[i][3], al[i][3]);
        }
#pragma unroll
        for (int j = 0; j < 2; j++) { // B fragment: (t, g), (t + 4, g)
            const float *Bc = B + (k0 + t) * LD + c0 + j * 8 + g;
            tf32_split(Bc[0], bh[j][0], bl[j][0]);
            tf32_split(Bc[4 * LD], bh[j][1], bl[j][1]);
        }
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 2; j++) {
                mma_tf32(acc[i][j], al[i], bh[j]);
                mma_tf32(acc[i][j], ah[i], bl[j]);
                mma_tf32(acc[i][j], ah[i], bh[j]);
            }
    }
}
// f(row, col, value) for every accumulator element this thread holds:
// (g, 2t), (g, 2t + 1), (g + 8, 2t), (g + 8, 2t + 1) of each 16 x 8 block
template <int KB, class F> __device__ __forceinline__ void tc_each(const TcAcc &acc, F f)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = (warp / (KB / 16)) * 32, c0 = (warp % (KB / 16)) * 16;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) f(r0 + i * 16 + g + (e >> 1) * 8, c0 + j * 8 + 2 * t + (e & 1), acc[i][j][e]);
}

// k_cr_odd with tensor-core products: S = I - Q P, M11 = S^{-1} (the Tile
// inverse), M10 = -M11 Q, M01 = -P M11, M00 = I - P M10.
template <int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_cr_odd_tc(const float *__restrict__ Pl, const float *__restrict__ Ql, int first, int stride, float *M,
                unsigned *err)
{
    constexpr int NT = NTOf<KB>::value, LD = TileLD<float, KB>::value;
    using TL = Tile<float, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    static_assert(NT == KB * KB / 16, "one warp per 32 x 16 output block");
    const int j = first + blockIdx.x * stride;
    float *Mj = M + (size_t)blockIdx.x * 4 * TS;
    extern __shared__ char smraw[];
    float *sP = (float *)smem_align(smraw), *sQ = sP + TL::ELEMS, *sH = sQ + TL::ELEMS;
    float *buf = sH + TL::ELEMS;
    TL t(threadIdx.x);
    typename TL::Reg a;
    TcAcc acc;
    ld<float, KB>(sP, Pl + (size_t)j * TS);
    ld<float, KB>(sQ, Ql + (size_t)j * TS);
    __syncthreads();
    tc_zero(acc);
    tc_mm<KB>(acc, sQ, sP);
    tc_each<KB>(acc, [&](int r, int c, float v) { sH[r * LD + c] = (r == c ? 1.f : 0.f) - v; }); // S
    __syncthreads();
    t.rload(a, sH);
    const bool ok = t.inverse(a, buf);
    if (!ok && threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
    __syncthreads();
    t.rstore(sH, a); // M11
    t.gstore(Mj + 3 * TS, a);
    __syncthreads();
    tc_zero(acc);
    tc_mm<KB>(acc, sH, sQ);
    tc_each<KB>(acc, [&](int r, int c, float v) { Mj[2 * TS + r * KB + c] = -v; }); // M10
    __syncthreads(); // every read of Q is done
    tc_each<KB>(acc, [&](int r, int c, float v) { sQ[r * LD + c] = -v; });
    tc_zero(acc);
    tc_mm<KB>(acc, sP, sH);
    tc_each<KB>(acc, [&](int r, int c, float v) { Mj[TS + r * KB + c] = -v; }); // M01
    __syncthreads();
    tc_zero(acc);
    tc_mm<KB>(acc, sP, sQ);
    tc_each<KB>(acc, [&](int r, int c, float v) { Mj[r * KB + c] = (r == c ? 1.f : 0.f) - v; }); // M00
}

// k_cr_even with tensor-core products: blockIdx.y picks the result
//   0: P' = P_i - X_i (M01 Y)_{i-1}   1: Q' = Q_i - Y_i (M10 X)_{i+1}
//   2: X' = -X_i (M00 X)_{i-1}        3: Y' = -Y_i (M11 Y)_{i+1}
template <int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_cr_even_tc(const float *__restrict__ Pl, const float *__restrict__ Ql, const float *__restrict__ Xl,
                 const float *__restrict__ Yl, const float *__restrict__ Ml, int cnt, float *Pn, float *Qn,
                 float *Xn, float *Yn)
{
    constexpr int NT = NTOf<KB>::value, LD = TileLD<float, KB>::value;
    using TL = Tile<float, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    const int i = 2 * blockIdx.x, a_out = blockIdx.x, which = blockIdx.y;
    const bool left = i - 1 >= 0, right = i + 1 < cnt;
    const bool has = (which == 0 || which == 2) ? left : right;
    const float *base = which == 0 ? Pl + (size_t)i * TS : which == 1 ? Ql + (size_t)i * TS : nullptr;
    float *out = (which == 0 ? Pn : which == 1 ? Qn : which == 2 ? Xn : Yn) + (size_t)a_out * TS;
    if (!has) { // no neighbour on this side: P' = P_i, Q' = Q_i, X' = Y' = 0
        for (int q = threadIdx.x; q < KB * KB; q += NT) out[q] = base ? base[q] : 0.f;
        return;
    }
    const float *Mnb = Ml + (size_t)(left && (which == 0 || which == 2) ? (i - 2) / 2 : i / 2) * 4 * TS;
    const float *Lt = (which == 0 || which == 2 ? Xl : Yl) + (size_t)i * TS;
    const float *Mq = Mnb + (size_t)(which == 0 ? 1 : which == 1 ? 2 : which == 2 ? 0 : 3) * TS;
    const float *Rt = (which == 0 || which == 3 ? Yl : Xl) + (size_t)(which == 0 || which == 2 ? i - 1 : i + 1) * TS;
    extern __shared__ char smraw[];
    float *sA = (float *)smem_align(smraw), *sB = sA + TL::ELEMS, *sC = sB + TL::ELEMS;
    ld<float, KB>(sA, Mq);
    ld<float, KB>(sB, Rt);
    __syncthreads();
    TcAcc acc;
    tc_zero(acc);
    tc_mm<KB>(acc, sA, sB);
    tc_each<KB>(acc, [&](int r, int c, float v) { sC[r * LD + c] = v; });
    __syncthreads();
    ld<float, KB>(sA, Lt);
    __syncthreads();
    tc_zero(acc);
    tc_mm<KB>(acc, sA, sC);
    tc_each<KB>(acc, [&](int r, int c, float v) { out[r * KB + c] = (base ? base[r * KB + c] : 0.f) - v; });
}

// ---------------------------------------------------------------- solve
// vectors: level block a holds 2KB rows; element (row q, column h) of block a
// at level offset off lives at g[h * stride + (off + a) * 2KB + q].

// y[r] = sum_k M[r][k] x[k]  for a KB x KB global tile and nr columns, via shared
template <class T, int KB>
__device__ T tile_row_dot(const T *sM, const T *sx, int r, int h, int RCP)
{
    T acc = sc_zero<T>();
    for (int k = 0; k < KB; k++) acc = madd(acc, sM[r * TileLD<T, KB>::value + k], sx[k * RCP + h]);
    return acc;
}

constexpr int RRC = 4; // right-hand sides per reduced-solve CTA (keeps static shared memory < 48 KB)

// forward reduction at level l: even i -> block i/2 of level l+1
//   g'^0 = g^0_i - X_i (M00 g^0 + M01 g^1)_{i-1}
//   g'^1 = g^1_i - Y_i (M10 g^0 + M11 g^1)_{i+1}
template <class T, int KB>
__global__ void __launch_bounds__(128)
    k_cr_fwd(const T *__restrict__ Xl, const T *__restrict__ Yl, const T *__restrict__ Ml, int cnt, T *g,
             long long stride, long long off_l, long long off_n, int nrhs)
{
    constexpr size_t TS = (size_t)KB * KB;
    const int i = 2 * blockIdx.x;
    const int h0 = blockIdx.y * RRC, nr = min(RRC, nrhs - h0);
    extern __shared__ char smraw[];
    T *sM = (T *)smem_align(smraw); // one tile (dynamic: a 128-row tile exceeds the static limit)
    __shared__ T sx[2 * KB * RRC], sw[KB * RRC];
    const bool left = i - 1 >= 0, right = i + 1 < cnt;
    T *gi = g + (off_l + i) * 2 * KB, *gn = g + (off_n + blockIdx.x) * 2 * KB;
    for (int half = 0; half < 2; half++) {
        const bool has = half == 0 ? left : right;
        const int nb = half == 0 ? i - 1 : i + 1;
        if (has) {
            const T *Mb = Ml + (size_t)(half == 0 ? (i - 2) / 2 : i / 2) * 4 * TS;
            __syncthreads();
            for (int q = threadIdx.x; q < 2 * KB * nr; q += blockDim.x) {
                const int rr = q % (2 * KB), h = q / (2 * KB);
                sx[rr * RRC + h] = g[(h0 + h) * stride + (off_l + nb) * 2 * KB + rr];
            }
            // w = M_{row half}(nb) * x : rows 0..KB-1 of [M00 M01] (half 0) or [M10 M11] (half 1)
            for (int q = threadIdx.x; q < KB * RRC; q += blockDim.x) sw[q] = sc_zero<T>();
            for (int part = 0; part < 2; part++) {
                __syncthreads();
                const T *Mt = Mb + (size_t)(half * 2 + part) * TS;
                copy_tile_g2s<T, KB, 128>(sM, Mt);
                __syncthreads();
                for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
                    const int r = q / nr, h = q - r * nr;
                    sw[r * RRC + h] = sw[r * RRC + h] + tile_row_dot<T, KB>(sM, sx + part * KB * RRC, r, h, RRC);
                }
            }
            __syncthreads();
            // subtract X_i w (half 0) or Y_i w (half 1) from the new block's half
            const T *Ct = (half == 0 ? Xl : Yl) + (size_t)i * TS;
            copy_tile_g2s<T, KB, 128>(sM, Ct);
            __syncthreads();
            for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
                const int r = q / nr, h = q - r * nr;
                const T v = gi[(h0 + h) * stride + half * KB + r];
                gn[(h0 + h) * stride + half * KB + r] = v - tile_row_dot<T, KB>(sM, sw, r, h, RRC);
            }
        } else {
            __syncthreads();
            for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
                const int r = q / nr, h = q - r * nr;
                gn[(h0 + h) * stride + half * KB + r] = gi[(h0 + h) * stride + half * KB + r];
            }
        }
    }
}

// u_j = M_j (g_j - [X_j u^0_{j-1}; Y_j u^1_{j+1}]) for odd j (or the top block,
// first = 0, with no neighbours), then even blocks copy u from the level above.
template <class T, int KB>
__global__ void __launch_bounds__(128)
    k_cr_bwd(const T *__restrict__ Xl, const T *__restrict__ Yl, const T *__restrict__ Ml, int cnt, const T *g, T *u,
             long long stride, long long off_l, long long off_n, int nrhs, int top)
{
    constexpr size_t TS = (size_t)KB * KB;
    const int h0 = blockIdx.y * RRC, nr = min(RRC, nrhs - h0);
    extern __shared__ char smraw[];
    T *sM = (T *)smem_align(smraw); // one tile
    __shared__ T sx[2 * KB * RRC], sw[2 * KB * RRC];
    if (!top && (blockIdx.x & 1) == 0) {
        // even block: copy from level l+1
        const int i = blockIdx.x;
        for (int q = threadIdx.x; q < 2 * KB * nr; q += blockDim.x) {
            const int rr = q % (2 * KB), h = q / (2 * KB);
            u[(h0 + h) * stride + (off_l + i) * 2 * KB + rr] = u[(h0 + h) * stride + (off_n + i / 2) * 2 * KB + rr];
        }
        return;
    }
    const int j = blockIdx.x;
    const T *Mj = Ml + (size_t)(top ? 0 : (j - 1) / 2) * 4 * TS;
    for (int q = threadIdx.x; q < 2 * KB * nr; q += blockDim.x) {
        const int rr = q % (2 * KB), h = q / (2 * KB);
        sx[rr * RRC + h] = g[(h0 + h) * stride + (off_l + j) * 2 * KB + rr];
    }
    if (!top) {
        for (int half = 0; half < 2; half++) {
            const int nb = half == 0 ? j - 1 : j + 1;
            if (nb < 0 || nb >= cnt) continue;
            __syncthreads();
            const T *Ct = (half == 0 ? Xl : Yl) + (size_t)j * TS;
            copy_tile_g2s<T, KB, 128>(sM, Ct);
            for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
                const int r = q / nr, h = q - r * nr;
                // even neighbours of an odd block: their values sit in the level above
                sw[r * RRC + h] = u[(h0 + h) * stride + (off_n + nb / 2) * 2 * KB + half * KB + r];
            }
            __syncthreads();
            for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
                const int r = q / nr, h = q - r * nr;
                sx[(half * KB + r) * RRC + h] = sx[(half * KB + r) * RRC + h] - tile_row_dot<T, KB>(sM, sw, r, h, RRC);
            }
        }
    }
    // u_j = M_j x : out rows half 0: M00 x0 + M01 x1; half 1: M10 x0 + M11 x1
    __syncthreads();
    for (int q = threadIdx.x; q < 2 * KB * RRC; q += blockDim.x) sw[q] = sc_zero<T>();
    for (int quad = 0; quad < 4; quad++) {
        __syncthreads();
        const T *Mt = Mj + (size_t)quad * TS;
        copy_tile_g2s<T, KB, 128>(sM, Mt);
        __syncthreads();
        const int oh = quad >> 1, ih = quad & 1;
        for (int q = threadIdx.x; q < KB * nr; q += blockDim.x) {
            const int r = q / nr, h = q - r * nr;
            sw[(oh * KB + r) * RRC + h] = sw[(oh * KB + r) * RRC + h] + tile_row_dot<T, KB>(sM, sx + ih * KB * RRC, r, h, RRC);
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 2 * KB * nr; q += blockDim.x) {
        const int rr = q % (2 * KB), h = q / (2 * KB);
        u[(h0 + h) * stride + (off_l + j) * 2 * KB + rr] = sw[rr * RRC + h];
    }
}

// level-0 right-hand side (factor precision) <- FP64 residual of R
template <class T>
__global__ void k_red_load(const typename HighOf<T>::type *__restrict__ res, T *g, long long NR, long long stride,
                           int nrhs)
{
    const long long tot = NR * nrhs;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < tot; q += (long long)gridDim.x * blockDim.x) {
        const long long h = q / NR, r = q - h * NR;
        g[h * stride + r] = cvt_fast<T, typename HighOf<T>::type>(res[q]);
    }
}

// u += du (FP64); first sweep sets u = du
template <class T>
__global__ void k_red_accum(const T *__restrict__ du, typename HighOf<T>::type *u, long long NR, long long stride,
                            int nrhs, int first)
{
    using H = typename HighOf<T>::type;
    const long long tot = NR * nrhs;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < tot; q += (long long)gridDim.x * blockDim.x) {
        const long long h = q / NR, r = q - h * NR;
        const H d = cvt_fast<H, T>(du[h * stride + r]);
        u[q] = first ? d : u[q] + d;
    }
}

// res = g - R u in FP64 with the level-0 quadrant blocks, one CTA per interface
template <class H, int KB>
__global__ void __launch_bounds__(128)
    k_red_resid(const H *__restrict__ RP, const H *__restrict__ RQ, const H *__restrict__ RX, const H *__restrict__ RY,
                const H *__restrict__ g, const H *__restrict__ u, H *res, int nif, int nrhs)
{
    constexpr size_t TS = (size_t)KB * KB;
    const int i = blockIdx.x;
    const long long NR = (long long)nif * 2 * KB;
    for (int q = threadIdx.x; q < 2 * KB * nrhs; q += blockDim.x) {
        const int h = q / (2 * KB), rr = q - h * 2 * KB;
        const H *uh = u + h * NR;
        const int r = rr % KB;
        H acc = g[h * NR + (long long)i * 2 * KB + rr] - uh[(long long)i * 2 * KB + rr];
        if (rr < KB) { // b-equation: P_i t + X_i b_{i-1}
            for (int c = 0; c < KB; c++) acc = msub(acc, RP[(size_t)i * TS + r * KB + c], uh[(long long)i * 2 * KB + KB + c]);
            if (i > 0)
                for (int c = 0; c < KB; c++) acc = msub(acc, RX[(size_t)i * TS + r * KB + c], uh[(long long)(i - 1) * 2 * KB + c]);
        } else { // t-equation: Q_i b + Y_i t_{i+2}
            for (int c = 0; c < KB; c++) acc = msub(acc, RQ[(size_t)i * TS + r * KB + c], uh[(long long)i * 2 * KB + c]);
            if (i + 1 < nif)
                for (int c = 0; c < KB; c++)
                    acc = msub(acc, RY[(size_t)i * TS + r * KB + c], uh[(long long)(i + 1) * 2 * KB + KB + c]);
        }
        res[h * NR + (long long)i * 2 * KB + rr] = acc;
    }
}

// ---------------------------------------------------------------- solve, one latency per level (KB 32, 64)
// The kernels above fetch their tiles one after another, each behind a
// __syncthreads, so a level costs several memory latencies.  Here a CTA asks
// for every tile it needs at once (cp.async), then each warp forms whole rows
// of the matrix-vector products: lanes run along k (conflict-free shared
// reads) and warp_tsum reduces a group of rows x right-hand sides together.
// Level 0 reads the FP64 right-hand side of R directly and accumulates the
// FP64 solution itself (no separate narrowing and accumulation launches).
constexpr int QNT = 256;       // threads per CTA (8 warps)
constexpr int QWARPS = QNT / 32;

template <class T, int KB, int NRC> struct QSolve {
    static constexpr size_t TS = (size_t)KB * KB;
    static constexpr int R = 2 * KB;             // rows of a level block
    static constexpr int RPW = R / QWARPS;       // rows per warp
    static constexpr int G = RPW * NRC <= 32 ? RPW : 32 / NRC; // rows per reduction group
    static constexpr int V = G * NRC;            // values per warp_tsum
    // 128-row tiles (64 KB each) are read from global memory where they lie,
    // coalesced along k; smaller ones are staged in shared memory
    static constexpr bool GT = KB >= 128;
    // six tiles (staged) and four 2KB-vectors per column
    static constexpr size_t bytes = (GT ? 0 : 6 * TS * sizeof(T)) + 4 * (size_t)R * NRC * sizeof(T) + 64;
    static_assert(KB % 32 == 0 && RPW % G == 0 && (V & (V - 1)) == 0 && V <= 32, "QSolve shape");
};

// element (row q, column h) of level block a: input g (FP64 at level 0)
template <class T, class H>
__device__ __forceinline__ T q_in(const void *g, bool l0, long long ld, long long a, int q, int h, int KB)
{
    const long long o = h * ld + a * 2 * KB + q;
    return l0 ? cvt_fast<T, H>(((const H *)g)[o]) : ((const T *)g)[o];
}

template <class T> __device__ __forceinline__ void q_tiles(T *s, const T *g, int ntiles, int KB)
{
    const int chunks = ntiles * KB * KB * (int)sizeof(T) / 16;
    for (int c = threadIdx.x; c < chunks; c += QNT) cp_async16((char *)s + 16 * c, (const char *)g + 16 * c);
}

// rows [r0, r0 + RPW) of out[q][h] = sum_k A(q, k) x[h][k], k < NK, for the
// rows of one warp; A(q, k) = At[q - qa][k] for k < KB and Bt[q - qa][k - KB]
// beyond (two row-major KB x KB tiles side by side).  emit(q, h, sum) is
// called once per (row, column) by one lane.
template <class T, int KB, int NRC, int NK, class Emit>
__device__ __forceinline__ void q_rows(const T *At, const T *Bt, int qa, const T *x, int r0, int nr, Emit emit)
{
    using Q = QSolve<T, KB, NRC>;
    constexpr int E = NK / 32;
    const int lane = threadIdx.x & 31;
    T xv[NRC][E];
#pragma unroll
    for (int h = 0; h < NRC; h++)
#pragma unroll
        for (int e = 0; e < E; e++) xv[h][e] = h < nr ? x[h * 2 * KB + lane + 32 * e] : sc_zero<T>();
#pragma unroll 1
    for (int g0 = 0; g0 < Q::RPW; g0 += Q::G) {
        T v[Q::V];
#pragma unroll
        for (int g = 0; g < Q::G; g++) {
            const int rr = r0 + g0 + g - qa;
            T m[E];
#pragma unroll
            for (int e = 0; e < E; e++) {
                const int k = lane + 32 * e;
                m[e] = k < KB ? At[rr * KB + k] : Bt[rr * KB + k - KB];
            }
#pragma unroll
            for (int h = 0; h < NRC; h++) {
                T acc = sc_zero<T>();
#pragma unroll
                for (int e = 0; e < E; e++) acc = madd(acc, m[e], xv[h][e]);
                v[g * NRC + h] = acc;
            }
        }
        const T sum = warp_tsum(v, lane);
        constexpr int SH = 5 - (Q::V == 1 ? 0 : Q::V == 2 ? 1 : Q::V == 4 ? 2 : Q::V == 8 ? 3 : Q::V == 16 ? 4 : 5);
        if ((lane & ((1 << SH) - 1)) == 0) {
            const int idx = lane >> SH, g = idx / NRC, h = idx - g * NRC;
            if (h < nr) emit(r0 + g0 + g, h, sum);
        }
    }
}

// Forward reduction, one CTA per even block i of level l:
//   g'_i = g_i - [X_i (M00 x0 + M01 x1)_{i-1} ; Y_i (M10 x0 + M11 x1)_{i+1}]
// g at level 0 is FP64 (gld = n_iface * 2KB); level l+1 goes to gn.
template <class T, int KB, int NRC>
__global__ void __launch_bounds__(QNT)
    k_crq_fwd(const T *__restrict__ Xl, const T *__restrict__ Yl, const T *__restrict__ Ml, int cnt, const void *gin,
              int l0, long long gld, long long off_l, T *gn, long long stride, long long off_n, int nrhs)
{
    using H = typename HighOf<T>::type;
    using Q = QSolve<T, KB, NRC>;
    constexpr size_t TS = Q::TS;
    const int i = 2 * blockIdx.x;
    const int h0 = blockIdx.y * NRC, nr = min(NRC, nrhs - h0);
    extern __shared__ char smraw[];
    T *sM = (T *)smem_align(smraw);               // [half][M_half0 | M_half1]: 4 tiles (staged)
    T *sC = sM + (Q::GT ? 0 : 4 * TS);            // X_i, Y_i (staged)
    T *sx = sC + (Q::GT ? 0 : 2 * TS);            // [half][h][2KB]: the neighbours' blocks
    T *sw = sx + 2 * NRC * 2 * KB;                // [half][h][2KB] (first KB used): w
    const bool has[2] = {i - 1 >= 0, i + 1 < cnt};
    const T *gM[2] = {has[0] ? Ml + (size_t)((i - 2) / 2) * 4 * TS : nullptr,       // M00, M01 of odd block i-1
                      has[1] ? Ml + (size_t)(i / 2) * 4 * TS + 2 * TS : nullptr};  // M10, M11 of odd block i+1
    const T *gC[2] = {Xl + (size_t)i * TS, Yl + (size_t)i * TS};
    if constexpr (!Q::GT) {
        if (has[0]) {
            q_tiles(sM, gM[0], 2, KB);
            q_tiles(sC, gC[0], 1, KB);
        }
        if (has[1]) {
            q_tiles(sM + 2 * TS, gM[1], 2, KB);
            q_tiles(sC + TS, gC[1], 1, KB);
        }
    }
    cp_async_commit();
    for (int q = threadIdx.x; q < 2 * NRC * 2 * KB; q += QNT) {
        const int half = q / (NRC * 2 * KB), rem = q - half * NRC * 2 * KB, h = rem / (2 * KB), k = rem - h * 2 * KB;
        sx[q] = has[half] && h < nr ? q_in<T, H>(gin, l0, gld, off_l + i + (half ? 1 : -1), k, h0 + h, KB)
                                    : sc_zero<T>();
    }
    cp_async_wait_all();
    __syncthreads();
    const int warp = threadIdx.x >> 5, r0 = warp * Q::RPW, half = r0 / KB;
    // w rows: half h of the neighbour's M times its block
    const T *tM = Q::GT ? gM[half] : sM + half * 2 * TS, *tC = Q::GT ? gC[half] : sC + half * TS;
    if (has[half])
        q_rows<T, KB, NRC, 2 * KB>(tM, tM + TS, half * KB, sx + half * NRC * 2 * KB, r0,
                                   nr, [&](int q, int h, T v) { sw[(half * NRC + h) * 2 * KB + q - half * KB] = v; });
    __syncthreads();
    T *gout = gn + (off_n + blockIdx.x) * 2 * KB;
    if (has[half]) {
        q_rows<T, KB, NRC, KB>(tC, tC, half * KB, sw + half * NRC * 2 * KB, r0, nr,
                               [&](int q, int h, T v) {
                                   gout[(h0 + h) * stride + q] = q_in<T, H>(gin, l0, gld, off_l + i, q, h0 + h, KB) - v;
                               });
    } else {
        for (int q = r0 + (threadIdx.x & 31); q < r0 + Q::RPW; q += 32)
            for (int h = 0; h < nr; h++) gout[(h0 + h) * stride + q] = q_in<T, H>(gin, l0, gld, off_l + i, q, h0 + h, KB);
    }
}

// Back substitution at level l (top = the single top block): odd j (and the
// top block) solve u_j = M_j (g_j - [X_j u0_{j-1} ; Y_j u1_{j+1}]) with the
// even neighbours' values from level l+1 (un); even j copy theirs from there.
// Level 0 writes the FP64 solution U (ld gld): U = d on the first refinement
// pass, U += d after.
template <class T, int KB, int NRC>
__global__ void __launch_bounds__(QNT)
    k_crq_bwd(const T *__restrict__ Xl, const T *__restrict__ Yl, const T *__restrict__ Ml, int cnt, const void *gin,
              int l0, long long gld, long long off_l, const T *un, long long off_n, T *u, long long stride, void *U,
              int first, int nrhs, int top)
{
    using H = typename HighOf<T>::type;
    using Q = QSolve<T, KB, NRC>;
    constexpr size_t TS = Q::TS;
    const int j = blockIdx.x;
    const int h0 = blockIdx.y * NRC, nr = min(NRC, nrhs - h0);
    auto put = [&](int q, int h, T v) {
        if (l0) {
            H *o = (H *)U + (h0 + h) * gld + (long long)j * 2 * KB + q;
            const H d = cvt_fast<H, T>(v);
            *o = first ? d : *o + d;
        } else {
            u[(h0 + h) * stride + (off_l + j) * 2 * KB + q] = v;
        }
    };
    if (!top && (j & 1) == 0) {
        for (int q = threadIdx.x; q < 2 * KB * nr; q += QNT) {
            const int h = q / (2 * KB), rr = q - h * 2 * KB;
            put(rr, h, un[(h0 + h) * stride + (off_n + j / 2) * 2 * KB + rr]);
        }
        return;
    }
    extern __shared__ char smraw[];
    T *sM = (T *)smem_align(smraw);    // M00 M01 M10 M11 (staged)
    T *sC = sM + (Q::GT ? 0 : 4 * TS); // X_j, Y_j (staged)
    T *sv = sC + (Q::GT ? 0 : 2 * TS); // [half][h][2KB] (first KB used): neighbour values
    T *ss = sv + 2 * NRC * 2 * KB;     // [h][2KB]: g_j minus the couplings
    const bool has[2] = {!top && j - 1 >= 0, !top && j + 1 < cnt};
    const T *gMj = Ml + (size_t)(top ? 0 : (j - 1) / 2) * 4 * TS;
    const T *gC[2] = {Xl + (size_t)j * TS, Yl + (size_t)j * TS};
    if constexpr (!Q::GT) {
        q_tiles(sM, gMj, 4, KB);
        if (has[0]) q_tiles(sC, gC[0], 1, KB);
        if (has[1]) q_tiles(sC + TS, gC[1], 1, KB);
    }
    cp_async_commit();
    for (int q = threadIdx.x; q < NRC * 2 * KB; q += QNT) {
        const int h = q / (2 * KB), k = q - h * 2 * KB;
        ss[q] = h < nr ? q_in<T, H>(gin, l0, gld, off_l + j, k, h0 + h, KB) : sc_zero<T>();
        const int half = k / KB, kk = k - half * KB; // the even neighbours sit in the level above
        sv[(half * NRC + h) * 2 * KB + kk] =
            has[half] && h < nr ? un[(h0 + h) * stride + (off_n + (j + (half ? 1 : -1)) / 2) * 2 * KB + half * KB + kk]
                                : sc_zero<T>();
    }
    cp_async_wait_all();
    __syncthreads();
    const int warp = threadIdx.x >> 5, r0 = warp * Q::RPW, half = r0 / KB;
    const T *tC = Q::GT ? gC[half] : sC + half * TS, *tM = (Q::GT ? gMj : sM) + half * 2 * TS;
    if (has[half])
        q_rows<T, KB, NRC, KB>(tC, tC, half * KB, sv + half * NRC * 2 * KB, r0, nr,
                               [&](int q, int h, T v) { ss[h * 2 * KB + q] = ss[h * 2 * KB + q] - v; });
    __syncthreads();
    q_rows<T, KB, NRC, 2 * KB>(tM, tM + TS, half * KB, ss, r0, nr, [&](int q, int h, T v) { put(q, h, v); });
}

// Small tiles (KB <= 16): the same one-latency levels, with PPC block pairs
// (or blocks) per 128-thread CTA and one thread per (row, column) output
// summing over k itself -- a level block's products are too small for a warp
// per row.
template <class T, int KB, int NRC> struct SSolve {
    static constexpr int TS = KB * KB;
    static constexpr int R = 2 * KB;
    static constexpr int UNIT = R * NRC;                     // threads per block pair
    static constexpr int PPC = 128 / UNIT > 0 ? 128 / UNIT : 1; // pairs per CTA
    static constexpr int NT = PPC * UNIT;
    static constexpr size_t PAIR = ((6 * TS + 4 * R * NRC) * sizeof(T) + 15) / 16 * 16; // smem per pair
    static constexpr size_t bytes = PPC * PAIR + 64;
    static_assert(UNIT <= 128, "SSolve shape");
};

template <class T, int KB, int NRC>
__global__ void __launch_bounds__(SSolve<T, KB, NRC>::NT)
    k_crs_fwd(const T *__restrict__ Xl, const T *__restrict__ Yl, const T *__restrict__ Ml, int cnt, const void *gin,
              int l0, long long gld, long long off_l, T *gn, long long stride, long long off_n, int nrhs)
{
    using H = typename HighOf<T>::type;
    using Q = SSolve<T, KB, NRC>;
    constexpr int TS = Q::TS, R = Q::R;
    const int slot = threadIdx.x / Q::UNIT, lt = threadIdx.x - slot * Q::UNIT;
    const int a = blockIdx.x * Q::PPC + slot; // the new block a <- even block i = 2a
    const int i = 2 * a;
    const bool live = i < cnt;
    const int h0 = blockIdx.y * NRC, nr = min(NRC, nrhs - h0);
    extern __shared__ char smraw[];
    T *sM = (T *)(smem_align(smraw) + slot * Q::PAIR); // [half][M_half0 | M_half1]
    T *sC = sM + 4 * TS;                                // X_i, Y_i
    T *sx = sC + 2 * TS;                                // [half][h][2KB]
    T *sw = sx + 2 * NRC * R;                           // [half][h][2KB] (first KB used)
    const bool has0 = live && i - 1 >= 0, has1 = live && i + 1 < cnt;
    // every tile of the CTA's pairs at once (each pair's UNIT threads copy its own)
    auto tiles = [&](T *dst, const T *src, int ntiles) {
        const int chunks = ntiles * TS * (int)sizeof(T) / 16;
        for (int c = lt; c < chunks; c += Q::UNIT) cp_async16((char *)dst + 16 * c, (const char *)src + 16 * c);
    };
    if (has0) {
        tiles(sM, Ml + (size_t)((i - 2) / 2) * 4 * TS, 2);
        tiles(sC, Xl + (size_t)i * TS, 1);
    }
    if (has1) {
        tiles(sM + 2 * TS, Ml + (size_t)(i / 2) * 4 * TS + 2 * TS, 2);
        tiles(sC + TS, Yl + (size_t)i * TS, 1);
    }
    cp_async_commit();
    for (int q = lt; q < 2 * NRC * R; q += Q::UNIT) {
        const int half = q / (NRC * R), rem = q - half * NRC * R, h = rem / R, k = rem - h * R;
        const bool has = half ? has1 : has0;
        sx[q] = has && h < nr ? q_in<T, H>(gin, l0, gld, off_l + i + (half ? 1 : -1), k, h0 + h, KB) : sc_zero<T>();
    }
    cp_async_wait_all();
    __syncthreads();
    const int q = lt / NRC, h = lt - q * NRC, half = q / KB, rr = q - half * KB;
    const bool has = half ? has1 : has0;
    if (has && h < nr) { // w = [M_h0 M_h1] x_nb, row rr of this half
        const T *M0 = sM + half * 2 * TS, *x = sx + (half * NRC + h) * R;
        T acc = sc_zero<T>();
#pragma unroll
        for (int k = 0; k < KB; k++) acc = madd(acc, M0[rr * KB + k], x[k]);
#pragma unroll
        for (int k = 0; k < KB; k++) acc = madd(acc, M0[TS + rr * KB + k], x[KB + k]);
        sw[(half * NRC + h) * R + rr] = acc;
    }
    __syncthreads();
    if (live && h < nr) {
        T v = q_in<T, H>(gin, l0, gld, off_l + i, q, h0 + h, KB);
        if (has) {
            const T *Ct = sC + half * TS, *w = sw + (half * NRC + h) * R;
#pragma unroll
            for (int k = 0; k < KB; k++) v = msub(v, Ct[rr * KB + k], w[k]);
        }
        gn[(h0 + h) * stride + (off_n + a) * 2 * KB + q] = v;
    }
}

template <class T, int KB, int NRC>
__global__ void __launch_bounds__(SSolve<T, KB, NRC>::NT)
    k_crs_bwd(const T *__restrict__ Xl, const T *__restrict__ Yl, const T *__restrict__ Ml, int cnt, const void *gin,
              int l0, long long gld, long long off_l, const T *un, long long off_n, T *u, long long stride, void *U,
              int first, int nrhs, int top)
{
    using H = typename HighOf<T>::type;
    using Q = SSolve<T, KB, NRC>;
    constexpr int TS = Q::TS, R = Q::R;
    const int slot = threadIdx.x / Q::UNIT, lt = threadIdx.x - slot * Q::UNIT;
    const int j = blockIdx.x * Q::PPC + slot;
    const bool live = j < cnt;
    const int h0 = blockIdx.y * NRC, nr = min(NRC, nrhs - h0);
    const int q = lt / NRC, h = lt - q * NRC, half = q / KB, rr = q - half * KB;
    auto put = [&](T v) {
        if (l0) {
            H *o = (H *)U + (h0 + h) * gld + (long long)j * 2 * KB + q;
            const H d = cvt_fast<H, T>(v);
            *o = first ? d : *o + d;
        } else {
            u[(h0 + h) * stride + (off_l + j) * 2 * KB + q] = v;
        }
    };
    const bool odd = live && (top || (j & 1));
    extern __shared__ char smraw[];
    T *sM = (T *)(smem_align(smraw) + slot * Q::PAIR); // M00 M01 M10 M11
    T *sC = sM + 4 * TS;                                // X_j, Y_j
    T *sv = sC + 2 * TS;                                // [half][h][2KB] (first KB used): neighbour values
    T *ss = sv + 2 * NRC * R;                           // [h][2KB]: g_j minus the couplings
    const bool has0 = odd && !top && j - 1 >= 0, has1 = odd && !top && j + 1 < cnt;
    auto tiles = [&](T *dst, const T *src, int ntiles) {
        const int chunks = ntiles * TS * (int)sizeof(T) / 16;
        for (int c = lt; c < chunks; c += Q::UNIT) cp_async16((char *)dst + 16 * c, (const char *)src + 16 * c);
    };
    if (odd) tiles(sM, Ml + (size_t)(top ? 0 : (j - 1) / 2) * 4 * TS, 4);
    if (has0) tiles(sC, Xl + (size_t)j * TS, 1);
    if (has1) tiles(sC + TS, Yl + (size_t)j * TS, 1);
    cp_async_commit();
    if (odd)
        for (int t = lt; t < NRC * R; t += Q::UNIT) {
            const int hh = t / R, k = t - hh * R, hf = k / KB, kk = k - hf * KB;
            const bool hs = hf ? has1 : has0;
            ss[t] = hh < nr ? q_in<T, H>(gin, l0, gld, off_l + j, k, h0 + hh, KB) : sc_zero<T>();
            sv[(hf * NRC + hh) * R + kk] =
                hs && hh < nr ? un[(h0 + hh) * stride + (off_n + (j + (hf ? 1 : -1)) / 2) * 2 * KB + hf * KB + kk]
                              : sc_zero<T>();
        }
    cp_async_wait_all();
    __syncthreads();
    if (live && !odd && h < nr) put(un[(h0 + h) * stride + (off_n + j / 2) * 2 * KB + q]); // even block: from above
    // (every thread, of even blocks and spare slots too, passes the barriers below)
    const bool hs = half ? has1 : has0;
    T sv_q = sc_zero<T>();
    if (odd && h < nr) {
        sv_q = ss[h * R + q];
        if (hs) {
            const T *Ct = sC + half * TS, *v = sv + (half * NRC + h) * R;
#pragma unroll
            for (int k = 0; k < KB; k++) sv_q = msub(sv_q, Ct[rr * KB + k], v[k]);
        }
    }
    __syncthreads();
    if (odd && h < nr) ss[h * R + q] = sv_q;
    __syncthreads();
    if (odd && h < nr) {
        const T *Mq = sM + half * 2 * TS, *x = ss + h * R; // [M_half0 M_half1] row rr
        T acc = sc_zero<T>();
#pragma unroll
        for (int k = 0; k < KB; k++) acc = madd(acc, Mq[rr * KB + k], x[k]);
#pragma unroll
        for (int k = 0; k < KB; k++) acc = madd(acc, Mq[TS + rr * KB + k], x[KB + k]);
        put(acc);
    }
}

template <class T, int KB, int NRC> int run_red_solve_s(spk_plan *P, int nrhs, int iters, cudaStream_t st)
{
    using H = typename HighOf<T>::type;
    using Q = SSolve<T, KB, NRC>;
    constexpr size_t TS = (size_t)KB * KB;
    const long long NR = (long long)P->n_iface * 2 * KB;
    const long long stride = P->crg_stride;
    T *cg = (T *)P->d_crg;
    T *cu = cg + stride * P->nrhs_max;
    const T *cX = (const T *)P->d_crX, *cY = (const T *)P->d_crY, *cM = (const T *)P->d_crM;
    const int L = P->cr_levels;
    const int hy = (nrhs + NRC - 1) / NRC;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_crs_fwd<T, KB, NRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q::bytes) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_crs_bwd<T, KB, NRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q::bytes) !=
                cudaSuccess)
            return SPK_ECUDA;
        attr = true;
    }
    for (int it = 0; it < iters; it++) {
        const H *res = it == 0 ? (const H *)P->d_g : (const H *)P->d_rr;
        for (int l = 0; l < L; l++) {
            const int cnt = P->cr_count[l], pairs = (cnt + 1) / 2;
            k_crs_fwd<T, KB, NRC><<<dim3((pairs + Q::PPC - 1) / Q::PPC, hy), Q::NT, Q::bytes, st>>>(
                cX + (size_t)P->cr_off[l] * TS, cY + (size_t)P->cr_off[l] * TS, cM + (size_t)P->cr_moff[l] * 4 * TS, cnt,
                l == 0 ? (const void *)res : (const void *)cg, l == 0, l == 0 ? NR : stride, P->cr_off[l], cg, stride,
                P->cr_off[l + 1], nrhs);
            P->launches++;
        }
        k_crs_bwd<T, KB, NRC><<<dim3(1, hy), Q::NT, Q::bytes, st>>>(
            nullptr, nullptr, cM + (size_t)P->cr_moff[L] * 4 * TS, 1, L == 0 ? (const void *)res : (const void *)cg,
            L == 0, L == 0 ? NR : stride, P->cr_off[L], nullptr, 0, cu, stride, P->d_u, it == 0, nrhs, 1);
        P->launches++;
        for (int l = L - 1; l >= 0; l--) {
            const int cnt = P->cr_count[l];
            k_crs_bwd<T, KB, NRC><<<dim3((cnt + Q::PPC - 1) / Q::PPC, hy), Q::NT, Q::bytes, st>>>(
                cX + (size_t)P->cr_off[l] * TS, cY + (size_t)P->cr_off[l] * TS, cM + (size_t)P->cr_moff[l] * 4 * TS, cnt,
                l == 0 ? (const void *)res : (const void *)cg, l == 0, l == 0 ? NR : stride, P->cr_off[l], cu,
                P->cr_off[l + 1], cu, stride, P->d_u, it == 0, nrhs, 0);
            P->launches++;
        }
        if (it + 1 < iters) {
            k_red_resid<H, KB><<<P->n_iface, 128, 0, st>>>((const H *)P->d_RP, (const H *)P->d_RQ, (const H *)P->d_RX,
                                                           (const H *)P->d_RY, (const H *)P->d_g, (const H *)P->d_u,
                                                           (H *)P->d_rr, P->n_iface, nrhs);
            P->launches++;
        }
        SPK_CHECK_LAUNCH();
    }
    return SPK_OK;
}

template <class T, int KB, int NRC> int run_red_solve_q(spk_plan *P, int nrhs, int iters, cudaStream_t st)
{
    using H = typename HighOf<T>::type;
    using Q = QSolve<T, KB, NRC>;
    constexpr size_t TS = (size_t)KB * KB;
    const long long NR = (long long)P->n_iface * 2 * KB;
    const long long stride = P->crg_stride;
    T *cg = (T *)P->d_crg;
    T *cu = cg + stride * P->nrhs_max;
    const T *cX = (const T *)P->d_crX, *cY = (const T *)P->d_crY, *cM = (const T *)P->d_crM;
    const int L = P->cr_levels;
    const int hy = (nrhs + NRC - 1) / NRC;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_crq_fwd<T, KB, NRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q::bytes) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_crq_bwd<T, KB, NRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q::bytes) !=
                cudaSuccess)
            return SPK_ECUDA;
        attr = true;
    }
    for (int it = 0; it < iters; it++) {
        const H *res = it == 0 ? (const H *)P->d_g : (const H *)P->d_rr;
        for (int l = 0; l < L; l++) {
            const int cnt = P->cr_count[l];
            k_crq_fwd<T, KB, NRC><<<dim3((cnt + 1) / 2, hy), QNT, Q::bytes, st>>>(
                cX + (size_t)P->cr_off[l] * TS, cY + (size_t)P->cr_off[l] * TS, cM + (size_t)P->cr_moff[l] * 4 * TS, cnt,
                l == 0 ? (const void *)res : (const void *)cg, l == 0, l == 0 ? NR : stride, P->cr_off[l], cg, stride,
                P->cr_off[l + 1], nrhs);
            P->launches++;
        }
        // the top block: level L (level 0 itself when R has one block)
        k_crq_bwd<T, KB, NRC><<<dim3(1, hy), QNT, Q::bytes, st>>>(
            nullptr, nullptr, cM + (size_t)P->cr_moff[L] * 4 * TS, 1, L == 0 ? (const void *)res : (const void *)cg,
            L == 0, L == 0 ? NR : stride, P->cr_off[L], nullptr, 0, cu, stride, P->d_u, it == 0, nrhs, 1);
        P->launches++;
        for (int l = L - 1; l >= 0; l--) {
            const int cnt = P->cr_count[l];
            k_crq_bwd<T, KB, NRC><<<dim3(cnt, hy), QNT, Q::bytes, st>>>(
                cX + (size_t)P->cr_off[l] * TS, cY + (size_t)P->cr_off[l] * TS, cM + (size_t)P->cr_moff[l] * 4 * TS, cnt,
                l == 0 ? (const void *)res : (const void *)cg, l == 0, l == 0 ? NR : stride, P->cr_off[l], cu,
                P->cr_off[l + 1], cu, stride, P->d_u, it == 0, nrhs, 0);
            P->launches++;
        }
        if (it + 1 < iters) {
            k_red_resid<H, KB><<<P->n_iface, 128, 0, st>>>((const H *)P->d_RP, (const H *)P->d_RQ, (const H *)P->d_RX,
                                                           (const H *)P->d_RY, (const H *)P->d_g, (const H *)P->d_u,
                                                           (H *)P->d_rr, P->n_iface, nrhs);
            P->launches++;
        }
        SPK_CHECK_LAUNCH();
    }
    return SPK_OK;
}

template <class T, int KB> int run_red_factor(spk_plan *P, cudaStream_t st)
{
    using S = RedSmem<T, KB>;
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t TS = (size_t)KB * KB;
    // FP32 factors with 64- or 128-row tiles: the block products on the tensor cores
    constexpr bool TC = std::is_same<T, float>::value && (KB == 64 || KB == 128);
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_cr_odd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bytes) != cudaSuccess ||
            cudaFuncSetAttribute(k_cr_even<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bytes) != cudaSuccess)
            return SPK_ECUDA;
        if constexpr (TC) {
            if (cudaFuncSetAttribute(k_cr_odd_tc<KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bytes) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_cr_even_tc<KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bytes) !=
                    cudaSuccess)
                return SPK_ECUDA;
        }
        attr = true;
    }
    auto odd = [&](const T *Pp, const T *Qp, int first, int stride, int count, T *Mo) {
        if constexpr (TC)
            k_cr_odd_tc<KB><<<count, NT, S::bytes, st>>>(Pp, Qp, first, stride, Mo, P->d_err);
        else
            k_cr_odd<T, KB><<<count, NT, S::bytes, st>>>(Pp, Qp, first, stride, Mo, P->d_err);
    };
    using H = typename HighOf<T>::type;
    const long long c0 = (long long)P->n_iface * TS;
    k_red_cvt<T><<<256, 256, 0, st>>>((const H *)P->d_RP, (T *)P->d_crP, c0);
    k_red_cvt<T><<<256, 256, 0, st>>>((const H *)P->d_RQ, (T *)P->d_crQ, c0);
    k_red_cvt<T><<<256, 256, 0, st>>>((const H *)P->d_RX, (T *)P->d_crX, c0);
    k_red_cvt<T><<<256, 256, 0, st>>>((const H *)P->d_RY, (T *)P->d_crY, c0);
    SPK_CHECK_LAUNCH();
    P->launches += 4;
    T *cP = (T *)P->d_crP, *cQ = (T *)P->d_crQ, *cX = (T *)P->d_crX, *cY = (T *)P->d_crY, *cM = (T *)P->d_crM;
    for (int l = 0; l < P->cr_levels; l++) {
        const int cnt = P->cr_count[l];
        const size_t o = (size_t)P->cr_off[l] * TS, on = (size_t)P->cr_off[l + 1] * TS;
        T *Ml = cM + (size_t)P->cr_moff[l] * 4 * TS;
        const int nodd = cnt / 2, neven = (cnt + 1) / 2;
        if (nodd > 0) {
            odd(cP + o, cQ + o, 1, 2, nodd, Ml);
            SPK_CHECK_LAUNCH();
        }
        if constexpr (TC)
            k_cr_even_tc<KB><<<dim3(neven, 4), NT, S::bytes, st>>>(cP + o, cQ + o, cX + o, cY + o, Ml, cnt, cP + on,
                                                                   cQ + on, cX + on, cY + on);
        else
            k_cr_even<T, KB><<<dim3(neven, 4), NT, S::bytes, st>>>(cP + o, cQ + o, cX + o, cY + o, Ml, cnt, cP + on,
                                                                   cQ + on, cX + on, cY + on);
        SPK_CHECK_LAUNCH();
        P->launches += 2;
    }
    // top: a single block
    {
        const int L = P->cr_levels;
        const size_t o = (size_t)P->cr_off[L] * TS;
        odd(cP + o, cQ + o, 0, 1, 1, cM + (size_t)P->cr_moff[L] * 4 * TS);
        SPK_CHECK_LAUNCH();
        P->launches++;
    }
    return SPK_OK;
}

template <class T, int KB> int run_red_solve(spk_plan *P, int nrhs, int iters, cudaStream_t st)
{
    if constexpr (KB == 32 || (KB == 64 && sizeof(T) <= 8) || (KB == 128 && sizeof(T) == 4)) {
        if (nrhs == 1) return run_red_solve_q<T, KB, 1>(P, nrhs, iters, st);
        return run_red_solve_q<T, KB, 4>(P, nrhs, iters, st);
    }
    if constexpr (KB <= 16 && KB * (int)sizeof(T) >= 16) { // a tile row of 16 bytes or more: cp.async-sized tiles
        if (nrhs == 1) return run_red_solve_s<T, KB, 1>(P, nrhs, iters, st);
        return run_red_solve_s<T, KB, 4>(P, nrhs, iters, st);
    }
    using H = typename HighOf<T>::type;
    constexpr size_t TS = (size_t)KB * KB;
    const long long NR = (long long)P->n_iface * 2 * KB;
    const long long stride = P->crg_stride;
    T *cg = (T *)P->d_crg;
    T *cu = cg + stride * P->nrhs_max;
    const T *cX = (const T *)P->d_crX, *cY = (const T *)P->d_crY, *cM = (const T *)P->d_crM;
    const int L = P->cr_levels;
    const dim3 blk(128);
    const int hy = (nrhs + RRC - 1) / RRC;
    constexpr size_t sm = RedSmem<T, KB>::solve;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_cr_fwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess ||
            cudaFuncSetAttribute(k_cr_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return SPK_ECUDA;
        attr = true;
    }
    for (int it = 0; it < iters; it++) {
        const H *res = it == 0 ? (const H *)P->d_g : (const H *)P->d_rr;
        k_red_load<T><<<256, 256, 0, st>>>(res, cg, NR, stride, nrhs);
        P->launches++;
        for (int l = 0; l < L; l++) {
            const int cnt = P->cr_count[l];
            k_cr_fwd<T, KB><<<dim3((cnt + 1) / 2, hy), blk, sm, st>>>(
                cX + (size_t)P->cr_off[l] * TS, cY + (size_t)P->cr_off[l] * TS, cM + (size_t)P->cr_moff[l] * 4 * TS, cnt, cg,
                stride, P->cr_off[l], P->cr_off[l + 1], nrhs);
            P->launches++;
        }
        k_cr_bwd<T, KB><<<dim3(1, hy), blk, sm, st>>>(nullptr, nullptr, cM + (size_t)P->cr_moff[L] * 4 * TS, 1, cg, cu, stride,
                                                     P->cr_off[L], 0, nrhs, 1);
        P->launches++;
        for (int l = L - 1; l >= 0; l--) {
            const int cnt = P->cr_count[l];
            k_cr_bwd<T, KB><<<dim3(cnt, hy), blk, sm, st>>>(cX + (size_t)P->cr_off[l] * TS, cY + (size_t)P->cr_off[l] * TS,
                                                           cM + (size_t)P->cr_moff[l] * 4 * TS, cnt, cg, cu, stride,
                                                           P->cr_off[l], P->cr_off[l + 1], nrhs, 0);
            P->launches++;
        }
        k_red_accum<T><<<256, 256, 0, st>>>(cu, (H *)P->d_u, NR, stride, nrhs, it == 0);
        P->launches++;
        if (it + 1 < iters) {
            k_red_resid<H, KB><<<P->n_iface, 128, 0, st>>>((const H *)P->d_RP, (const H *)P->d_RQ, (const H *)P->d_RX,
                                                           (const H *)P->d_RY, (const H *)P->d_g, (const H *)P->d_u,
                                                           (H *)P->d_rr, P->n_iface, nrhs);
            P->launches++;
        }
        SPK_CHECK_LAUNCH();
    }
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

template <class T> int disp_rf(spk_plan *P, cudaStream_t st) { SPK_KB_SWITCH(run_red_factor, T, P, st) }
template <class T> int disp_rs(spk_plan *P, int nrhs, int it, cudaStream_t st) { SPK_KB_SWITCH(run_red_solve, T, P, nrhs, it, st) }

} // namespace

extern "C" int spk_reduced_factor(spk_plan *P, void *stream)
{
    if (P->n_iface <= 0) return SPK_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const bool low = P->mode == SPK_MIXED && !P->red_fp64; // factor-precision cyclic reduction
    if (P->is_complex) return low ? disp_rf<cfloat>(P, st) : disp_rf<cdouble>(P, st);
    return low ? disp_rf<float>(P, st) : disp_rf<double>(P, st);
}

extern "C" int spk_reduced_solve(spk_plan *P, int nrhs, int refine_iters, void *stream)
{
    if (P->n_iface <= 0) return SPK_OK;
    if (refine_iters < 1) refine_iters = 1;
    cudaStream_t st = (cudaStream_t)stream;
    const bool low = P->mode == SPK_MIXED && !P->red_fp64;
    if (P->is_complex)
        return low ? disp_rs<cfloat>(P, nrhs, refine_iters, st) : disp_rs<cdouble>(P, nrhs, refine_iters, st);
    return low ? disp_rs<float>(P, nrhs, refine_iters, st) : disp_rs<double>(P, nrhs, refine_iters, st);
}
