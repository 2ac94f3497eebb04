// spike_common.cuh -- scalar types and KB x KB tile operations shared by the
// SPIKE kernels (sm_103a).
//
// Every dense block of the block-tridiagonal view of A_i is a KB x KB tile.
// A CTA of NT threads owns one tile operation at a time; each active thread
// holds a contiguous TR x TC register sub-tile, so operand fetches are
// 8/16-byte vectors.  Shared tiles have row stride TileLD (KB + 16 bytes).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "spike_internal.h"

// ---------------------------------------------------------------- scalars
struct cfloat {
    float re, im;
};
struct cdouble {
    double re, im;
};

#define SPK_HD __host__ __device__ __forceinline__

SPK_HD cfloat operator+(cfloat a, cfloat b) { return {a.re + b.re, a.im + b.im}; }
SPK_HD cfloat operator-(cfloat a, cfloat b) { return {a.re - b.re, a.im - b.im}; }
SPK_HD cfloat operator-(cfloat a) { return {-a.re, -a.im}; }
SPK_HD cfloat operator*(cfloat a, cfloat b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
SPK_HD cdouble operator+(cdouble a, cdouble b) { return {a.re + b.re, a.im + b.im}; }
SPK_HD cdouble operator-(cdouble a, cdouble b) { return {a.re - b.re, a.im - b.im}; }
SPK_HD cdouble operator-(cdouble a) { return {-a.re, -a.im}; }
SPK_HD cdouble operator*(cdouble a, cdouble b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// acc + a*b
SPK_HD float madd(float acc, float a, float b) { return fmaf(a, b, acc); }
SPK_HD double madd(double acc, double a, double b) { return fma(a, b, acc); }
SPK_HD cfloat madd(cfloat acc, cfloat a, cfloat b)
{
    return {fmaf(-a.im, b.im, fmaf(a.re, b.re, acc.re)), fmaf(a.im, b.re, fmaf(a.re, b.im, acc.im))};
}
SPK_HD cdouble madd(cdouble acc, cdouble a, cdouble b)
{
    return {fma(-a.im, b.im, fma(a.re, b.re, acc.re)), fma(a.im, b.re, fma(a.re, b.im, acc.im))};
}
// acc - a*b
SPK_HD float msub(float acc, float a, float b) { return fmaf(-a, b, acc); }
SPK_HD double msub(double acc, double a, double b) { return fma(-a, b, acc); }
SPK_HD cfloat msub(cfloat acc, cfloat a, cfloat b) { return madd(acc, -a, b); }
SPK_HD cdouble msub(cdouble acc, cdouble a, cdouble b) { return madd(acc, -a, b); }

template <class T> SPK_HD T sc_zero() { return T(0); }
template <> SPK_HD cfloat sc_zero<cfloat>() { return {0.f, 0.f}; }
template <> SPK_HD cdouble sc_zero<cdouble>() { return {0.0, 0.0}; }
template <class T> SPK_HD T sc_one() { return T(1); }
template <> SPK_HD cfloat sc_one<cfloat>() { return {1.f, 0.f}; }
template <> SPK_HD cdouble sc_one<cdouble>() { return {1.0, 0.0}; }

SPK_HD float sc_recip(float a) { return 1.0f / a; }
SPK_HD double sc_recip(double a) { return 1.0 / a; }
SPK_HD cfloat sc_recip(cfloat a)
{
    float s = 1.0f / (a.re * a.re + a.im * a.im);
    return {a.re * s, -a.im * s};
}
SPK_HD cdouble sc_recip(cdouble a)
{
    double s = 1.0 / (a.re * a.re + a.im * a.im);
    return {a.re * s, -a.im * s};
}
// correctly rounded reciprocal without the IEEE-division slow path
__device__ __forceinline__ float sc_frcp(float a) { return __frcp_rn(a); }
__device__ __forceinline__ double sc_frcp(double a) { return __drcp_rn(a); }
__device__ __forceinline__ cfloat sc_frcp(cfloat a)
{
    const float s = __frcp_rn(fmaf(a.re, a.re, a.im * a.im));
    return {a.re * s, -a.im * s};
}
__device__ __forceinline__ cdouble sc_frcp(cdouble a)
{
    const double s = __drcp_rn(fma(a.re, a.re, a.im * a.im));
    return {a.re * s, -a.im * s};
}
// reciprocal for the factor-precision inverse: FP32 uses the hardware
// approximation refined by one Newton step (within 1 ulp; the refinement
// absorbs it), FP64 the correctly rounded one.
__device__ __forceinline__ float sc_rcp_fast(float a)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    const float e = fmaf(-a, r, 1.0f);
    return fmaf(r, e, r);
}
__device__ __forceinline__ double sc_rcp_fast(double a) { return __drcp_rn(a); }
__device__ __forceinline__ cfloat sc_rcp_fast(cfloat a)
{
    const float s = sc_rcp_fast(fmaf(a.re, a.re, a.im * a.im));
    return {a.re * s, -a.im * s};
}
__device__ __forceinline__ cdouble sc_rcp_fast(cdouble a) { return sc_frcp(a); }
SPK_HD double sc_abs2(float a) { return (double)a * a; }
SPK_HD double sc_abs2(double a) { return a * a; }
SPK_HD double sc_abs2(cfloat a) { return (double)a.re * a.re + (double)a.im * a.im; }
SPK_HD double sc_abs2(cdouble a) { return a.re * a.re + a.im * a.im; }
SPK_HD bool sc_finite_nonzero(float a) { return a != 0.f && isfinite(a); }
SPK_HD bool sc_finite_nonzero(double a) { return a != 0.0 && isfinite(a); }
SPK_HD bool sc_finite_nonzero(cfloat a) { return (a.re != 0.f || a.im != 0.f) && isfinite(a.re) && isfinite(a.im); }
SPK_HD bool sc_finite_nonzero(cdouble a) { return (a.re != 0.0 || a.im != 0.0) && isfinite(a.re) && isfinite(a.im); }

// conversions between the FP64 ("high") type and the factor type
template <class T, class H> SPK_HD T sc_cvt(H v);
template <> SPK_HD float sc_cvt<float, double>(double v) { return (float)v; }
template <> SPK_HD double sc_cvt<double, double>(double v) { return v; }
template <> SPK_HD cfloat sc_cvt<cfloat, cdouble>(cdouble v) { return {(float)v.re, (float)v.im}; }
template <> SPK_HD cdouble sc_cvt<cdouble, cdouble>(cdouble v) { return v; }
template <> SPK_HD double sc_cvt<double, float>(float v) { return v; }
template <> SPK_HD cdouble sc_cvt<cdouble, cfloat>(cfloat v) { return {v.re, v.im}; }

// High (FP64) type matching a factor type
template <class T> struct HighOf;
template <> struct HighOf<float> { using type = double; };
template <> struct HighOf<double> { using type = double; };
template <> struct HighOf<cfloat> { using type = cdouble; };
template <> struct HighOf<cdouble> { using type = cdouble; };

// threads per CTA for a tile size
template <int KB> struct NTOf {
    static constexpr int value = KB >= 128 ? 1024 : KB >= 64 ? 256 : KB == 32 ? 128 : KB == 16 ? 64 : 32;
};

// ------------------------------------------------------------ vector access
// N contiguous elements (N in {1, 2} or a multiple of 4) between registers and memory in
// 8- or 16-byte transactions.  The pointer must be aligned to
// min(16, N * sizeof(T)) bytes.
template <class T> __device__ __forceinline__ T from_f2(float x, float y);
template <> __device__ __forceinline__ double from_f2<double>(float x, float y)
{
    return __hiloint2double(__float_as_int(y), __float_as_int(x));
}
template <> __device__ __forceinline__ cfloat from_f2<cfloat>(float x, float y) { return {x, y}; }
__device__ __forceinline__ float2 to_f2(double d)
{
    return make_float2(__int_as_float(__double2loint(d)), __int_as_float(__double2hiint(d)));
}
__device__ __forceinline__ float2 to_f2(cfloat c) { return make_float2(c.re, c.im); }

template <class T, int N> __device__ __forceinline__ void vld(T (&d)[N], const T *p)
{
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
        for (int q = 0; q < N / 4; q++) {
            const float4 v = reinterpret_cast<const float4 *>(p)[q];
            d[4 * q] = v.x; d[4 * q + 1] = v.y; d[4 * q + 2] = v.z; d[4 * q + 3] = v.w;
        }
    } else if constexpr (sizeof(T) == 4 && N == 2) {
        const float2 v = *reinterpret_cast<const float2 *>(p);
        d[0] = v.x; d[1] = v.y;
    } else if constexpr (sizeof(T) == 8 && N >= 2) {
#pragma unroll
        for (int q = 0; q < N / 2; q++) {
            const float4 v = reinterpret_cast<const float4 *>(p)[q];
            d[2 * q] = from_f2<T>(v.x, v.y);
            d[2 * q + 1] = from_f2<T>(v.z, v.w);
        }
    } else {
#pragma unroll
        for (int q = 0; q < N; q++) d[q] = p[q];
    }
}
template <class T, int N> __device__ __forceinline__ void vst(T *p, const T (&d)[N])
{
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
        for (int q = 0; q < N / 4; q++)
            reinterpret_cast<float4 *>(p)[q] = make_float4(d[4 * q], d[4 * q + 1], d[4 * q + 2], d[4 * q + 3]);
    } else if constexpr (sizeof(T) == 4 && N == 2) {
        *reinterpret_cast<float2 *>(p) = make_float2(d[0], d[1]);
    } else if constexpr (sizeof(T) == 8 && N >= 2) {
#pragma unroll
        for (int q = 0; q < N / 2; q++) {
            const float2 a = to_f2(d[2 * q]), b = to_f2(d[2 * q + 1]);
            reinterpret_cast<float4 *>(p)[q] = make_float4(a.x, a.y, b.x, b.y);
        }
    } else {
#pragma unroll
        for (int q = 0; q < N; q++) p[q] = d[q];
    }
}

// shared-memory row stride of a KB x KB tile: 16 bytes of padding keeps every
// row 16-byte aligned and shifts consecutive rows across banks
template <class T, int KB> struct TileLD {
    static constexpr int value = KB + (16 / (int)sizeof(T) > 0 ? 16 / (int)sizeof(T) : 1);
};

// ------------------------------------------------------------ tile geometry
// Thread (tx, ty) owns the contiguous TR x TC sub-tile at rows ty*TR + i,
// columns tx*TC + j.  Operand fetches are vectors: a row-major right operand
// gives TC contiguous elements per k, a left operand stored transposed
// (column-major, "At") gives TR contiguous elements per k.
template <class T, int KB, int NT> struct Tile {
    // 128-row tiles: a 32 x 32 thread grid keeps every sub-tile 4 x 4
    static constexpr int TX = KB < 16 ? KB : KB >= 128 ? 32 : 16;
    static constexpr int TY0 = NT / TX;
    static constexpr int TY = TY0 < KB ? TY0 : KB;
    static constexpr int TC = KB / TX;
    static constexpr int TR = KB / TY;
    static constexpr int LD = TileLD<T, KB>::value; // shared-memory row stride
    static constexpr int ELEMS = KB * LD;           // shared-memory tile size
    static constexpr int ACTIVE = TX * TY;          // threads that own a sub-tile
    // the blocked inverse runs when every thread owns a 4 x 4 sub-tile
    // every thread owns 4 columns and a multiple of 4 rows; pivot block q is
    // columns 4q..4q+3 of thread column tx = q
    static constexpr bool BLOCK4 = (TC == 4 && TR % 4 == 0 && TR <= 8 && TX == KB / 4);
    static constexpr int RB = TR / 4; // pivot-block rows per thread
    static constexpr int INV_HALF = 12 * KB + 16;  // pivot columns + P^{-1} + V' + pivot rows
    static constexpr int INV_BUF = BLOCK4 ? 2 * INV_HALF + KB : 4 * KB; // shared scratch elements for inverse()

    // Warp footprint: where the grid allows it, a warp's 32 lanes cover 8
    // sub-tile columns x 4 sub-tile rows (32 x 16 elements with 4 x 4
    // sub-tiles), so one k step of a product reads 64 B of the left operand
    // and 128 B of the right one -- two shared-memory wavefronts per 16 FMAs
    // per thread, where a 16 x 2 footprint needs three.
    static constexpr bool SQ = NT % 32 == 0 && ACTIVE == NT && TX % 8 == 0 && TY % 4 == 0;
    static constexpr int WX = SQ ? 8 : TX;  // sub-tile columns per warp
    static constexpr int WY = SQ ? 4 : 32 / (TX < 32 ? TX : 32); // sub-tile rows per warp

    using Reg = T[TR][TC];

    int tx, ty;
    int wr0, wr1; // rows [wr0, wr1) of the tile are owned by this thread's warp
    int wc0, wc1; // and columns [wc0, wc1)
    bool act;
    __device__ __forceinline__ Tile(int tid)
    {
        act = tid < ACTIVE;
        if constexpr (SQ) {
            const int warp = tid >> 5, lane = tid & 31;
            constexpr int WPR = TX / WX; // warps per row of sub-tiles
            tx = (warp % WPR) * WX + (lane % WX);
            ty = (warp / WPR) * WY + (lane / WX);
            wr0 = (warp / WPR) * WY * TR;
            wr1 = wr0 + WY * TR;
            wc0 = (warp % WPR) * WX * TC;
            wc1 = wc0 + WX * TC;
        } else {
            tx = tid % TX;
            ty = tid / TX;
            wr0 = ((tid & ~31) / TX) * TR;          // first row of the warp
            wr1 = ((tid | 31) / TX) * TR + TR;      // one past its last row
            wc0 = 0;
            wc1 = KB;
        }
        if (wr1 > KB) wr1 = KB;
    }
    __device__ __forceinline__ int row(int i) const { return ty * TR + i; }
    __device__ __forceinline__ int col(int j) const { return tx * TC + j; }

    __device__ __forceinline__ void rzero(Reg &a) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) a[i][j] = sc_zero<T>();
    }
    // register tile <- shared tile (threads without a sub-tile hold zeros)
    __device__ __forceinline__ void rload(Reg &a, const T *s) const
    {
        if (!act) {
            rzero(a);
            return;
        }
#pragma unroll
        for (int i = 0; i < TR; i++) vld<T, TC>(a[i], s + row(i) * LD + col(0));
    }
    // shared tile <- register tile
    __device__ __forceinline__ void rstore(T *s, const Reg &a) const
    {
        if (!act) return;
#pragma unroll
        for (int i = 0; i < TR; i++) vst<T, TC>(s + row(i) * LD + col(0), a[i]);
    }
    // shared tile, transposed (column-major: element (r, c) at c*LD + r) <- register tile
    __device__ __forceinline__ void rstore_t(T *s, const Reg &a) const
    {
        if (!act) return;
#pragma unroll
        for (int j = 0; j < TC; j++) {
            T c[TR];
#pragma unroll
            for (int i = 0; i < TR; i++) c[i] = a[i][j];
            vst<T, TR>(s + col(j) * LD + row(0), c);
        }
    }
    // register tile <- dense global tile (row-major, ld KB)
    __device__ __forceinline__ void gload(Reg &a, const T *g) const
    {
        if (!act) {
            rzero(a);
            return;
        }
#pragma unroll
        for (int i = 0; i < TR; i++) vld<T, TC>(a[i], g + row(i) * KB + col(0));
    }
    // dense global tile (row-major, ld KB) <- register tile
    __device__ __forceinline__ void gstore(T *g, const Reg &a) const
    {
        if (!act) return;
#pragma unroll
        for (int i = 0; i < TR; i++) vst<T, TC>(g + row(i) * KB + col(0), a[i]);
    }
    // dense global tile, column-major (element (r, c) at c*KB + r) <- register tile
    __device__ __forceinline__ void gstore_t(T *g, const Reg &a) const
    {
        if (!act) return;
#pragma unroll
        for (int j = 0; j < TC; j++) {
            T c[TR];
#pragma unroll
            for (int i = 0; i < TR; i++) c[i] = a[i][j];
            vst<T, TR>(g + col(j) * KB + row(0), c);
        }
    }
    // acc (+|-)= A * B, A row-major in shared memory (scalar fetches)
    template <bool SUB> __device__ __forceinline__ void mm_rowA(Reg &acc, const T *A, const T *B) const
    {
        if (!act) return;
#pragma unroll 4
        for (int k = 0; k < KB; k++) {
            T a[TR], b[TC];
#pragma unroll
            for (int i = 0; i < TR; i++) a[i] = A[row(i) * LD + k];
            vld<T, TC>(b, B + k * LD + col(0));
#pragma unroll
            for (int i = 0; i < TR; i++)
#pragma unroll
                for (int j = 0; j < TC; j++) acc[i][j] = SUB ? msub(acc[i][j], a[i], b[j]) : madd(acc[i][j], a[i], b[j]);
        }
    }
    // acc (+|-)= A * B with A given transposed (At, column-major): vector fetches.
    // TRI = 1: A is upper triangular, 2: A lower triangular, 3: B lower
    // triangular, 4: B upper triangular -- the k range where the warp's rows
    // of A (columns of B) are zero is skipped (warp-uniform bounds, so only
    // exact zeros are left out and the result is unchanged).  LDA / LDB: row
    // strides of the two shared operands (LD for a padded tile, KB for a dense
    // one that arrived by a single bulk copy).
    template <bool SUB, int TRI = 0, int LDA = LD, int LDB = LD>
    __device__ __forceinline__ void mm_tA(Reg &acc, const T *At, const T *B) const
    {
        if (!act) return;
        const int k0 = TRI == 1 ? wr0 : TRI == 3 ? wc0 : 0;
        const int k1 = TRI == 2 ? wr1 : TRI == 4 ? wc1 : KB;
#pragma unroll 4
        for (int k = k0; k < k1; k++) {
            T a[TR], b[TC];
            vld<T, TR>(a, At + k * LDA + row(0));
            vld<T, TC>(b, B + k * LDB + col(0));
#pragma unroll
            for (int i = 0; i < TR; i++)
#pragma unroll
                for (int j = 0; j < TC; j++) acc[i][j] = SUB ? msub(acc[i][j], a[i], b[j]) : madd(acc[i][j], a[i], b[j]);
        }
    }
    __device__ __forceinline__ void mma(Reg &acc, const T *A, const T *B) const { mm_rowA<false>(acc, A, B); }
    __device__ __forceinline__ void mms(Reg &acc, const T *A, const T *B) const { mm_rowA<true>(acc, A, B); }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mma_t(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<false, 0, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mms_t(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 0, LDA, LDB>(acc, At, B);
    }
    // A upper triangular (acc += A B) / lower triangular (acc -= A B)
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mma_tu(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<false, 1, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mms_tl(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 2, LDA, LDB>(acc, At, B);
    }
    // A lower triangular (acc += A B) / upper triangular (acc -= A B)
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mma_tl(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<false, 2, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mms_tu(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 1, LDA, LDB>(acc, At, B);
    }
    // acc -= A B with B lower / upper triangular
    template <int LDA = LD, int LDB = LD>
    __device__ __forceinline__ void mms_t_bl(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 3, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD>
    __device__ __forceinline__ void mms_t_bu(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 4, LDA, LDB>(acc, At, B);
    }

    // In-place Gauss-Jordan inverse of the register tile, no pivoting (the
    // diagonal blocks of a diagonally dominant A stay diagonally dominant
    // under block elimination).  Step j, with p = S[j][j], a = column j and
    // b = row j:
    //     S[r][c] <- S[r][c] - a[r] b[c] / p     r != j, c != j
    //     S[j][c] <- b[c] / p,   S[r][j] <- -a[r] / p,   S[j][j] <- 1 / p
    // The owners of row j / column j publish them as vectors into a double-
    // buffered shared scratch, so each pivot costs one barrier; every element
    // then takes one FMA, and only the owners of row j / column j patch it.
    // buf: INV_BUF elements of shared memory (16-byte aligned).  All NT
    // threads must call.  Returns false in every thread if a pivot was zero
    // or not finite.
    __device__ __forceinline__ bool inverse(Reg &s, T *buf) const
    {
        if constexpr (BLOCK4)
            return inverse_b4(s, buf);
        else
            return inverse_r1(s, buf);
    }

    // Blocked Gauss-Jordan with 4 x 4 pivot blocks, each the sub-tile of one
    // thread.  With P the pivot block, U the pivot columns, B the pivot rows,
    // every element takes the same update
    //     S <- S - U' V',  U' = U - I (on the pivot rows),  V' = P^{-1} (B + I (on the pivot columns))
    // which yields P^{-1} on the pivot block, P^{-1} B on the pivot rows,
    // -U P^{-1} on the pivot columns and S - U P^{-1} B elsewhere.  Rows are
    // scaled to a unit diagonal first (and the inverse's columns back after),
    // so the pivot blocks stay O(1) and the I terms cancel nothing large.
    // Per 4 pivots: the pivot owner inverts P, every thread forms one element
    // of V', everyone applies 64 FMAs; two barriers.
    __device__ __forceinline__ bool inverse_b4(Reg &s, T *buf) const
    {
        bool ok = true;
        T *dg = buf + 2 * INV_HALF; // diagonal
        // the thread whose columns tx*4..tx*4+3 cross its rows holds those diagonal entries
        if (act && (RB == 1 ? tx == ty : (tx * 4) / TR == ty)) {
            const int o = RB == 1 ? 0 : tx * 4 - ty * TR;
            T d[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                d[j] = s[0][j];
#pragma unroll
                for (int i = 1; i < TR; i++) d[j] = (i == o + j) ? s[i][j] : d[j];
            }
            vst<T, 4>(dg + col(0), d);
        }
        __syncthreads();
        if (act) {
            T dr[TR];
            vld<T, TR>(dr, dg + row(0));
#pragma unroll
            for (int i = 0; i < TR; i++) {
                if (!sc_finite_nonzero(dr[i])) ok = false;
                const T rr = sc_rcp_fast(dr[i]);
#pragma unroll
                for (int jj = 0; jj < 4; jj++) s[i][jj] = s[i][jj] * rr;
            }
        }
        for (int q = 0; q < KB / 4; q++) {
            T *cbuf = buf + (q & 1) * INV_HALF; // [KB][4] pivot columns U'
            T *pbuf = cbuf + 4 * KB;            // [4][4] P^{-1}
            T *vbuf = pbuf + 16;                // [4][KB] V'
            T *rbuf = vbuf + 4 * KB;            // [4][KB] pivot rows B + I
            const bool rown = act && (RB == 1 ? ty == q : ty == (4 * q) / TR), cown = act && tx == q;
            const int ro = RB == 1 ? 0 : 4 * (q % RB); // first pivot row within the owner's rows
            if (rown) {
#pragma unroll
                for (int rb = 0; rb < RB; rb++)
                    if (ro == 4 * rb) {
#pragma unroll
                        for (int a = 0; a < 4; a++) {
                            T bb[4];
#pragma unroll
                            for (int jj = 0; jj < 4; jj++)
                                bb[jj] = (cown && a == jj) ? s[4 * rb + a][jj] + sc_one<T>() : s[4 * rb + a][jj];
                            vst<T, 4>(rbuf + a * KB + col(0), bb);
                        }
                    }
            }
            if (cown) {
#pragma unroll
                for (int i = 0; i < TR; i++) {
                    T u[4];
#pragma unroll
                    for (int t = 0; t < 4; t++) u[t] = (rown && i - ro == t) ? s[i][t] - sc_one<T>() : s[i][t];
                    vst<T, 4>(cbuf + row(i) * 4, u);
                }
                if (rown) { // pivot owner: P^{-1} by unblocked Gauss-Jordan in registers
#pragma unroll
                    for (int rb = 0; rb < RB; rb++)
                        if (ro == 4 * rb) {
                            T pinv[4][4];
#pragma unroll
                            for (int a = 0; a < 4; a++)
#pragma unroll
                                for (int b = 0; b < 4; b++) pinv[a][b] = s[4 * rb + a][b];
#pragma unroll
                            for (int k = 0; k < 4; k++) {
                                const T piv = pinv[k][k];
                                if (!sc_finite_nonzero(piv)) ok = false;
                                const T pr = sc_rcp_fast(piv);
#pragma unroll
                                for (int b = 0; b < 4; b++)
                                    if (b != k) pinv[k][b] = pinv[k][b] * pr;
#pragma unroll
                                for (int a = 0; a < 4; a++)
                                    if (a != k) {
                                        const T f = pinv[a][k];
#pragma unroll
                                        for (int b = 0; b < 4; b++)
                                            if (b != k) pinv[a][b] = msub(pinv[a][b], f, pinv[k][b]);
                                        pinv[a][k] = -(f * pr);
                                    }
                                pinv[k][k] = pr;
                            }
#pragma unroll
                            for (int a = 0; a < 4; a++) vst<T, 4>(pbuf + 4 * a, pinv[a]);
                        }
                }
            }
            __syncthreads();
            // V' = P^{-1} (B + I on the pivot columns), one element per thread
            for (int e = threadIdx.x; e < 4 * KB; e += NT) {
                const int tt = e / KB, c = e - tt * KB;
                T acc = sc_zero<T>();
#pragma unroll
                for (int a = 0; a < 4; a++) acc = madd(acc, pbuf[4 * tt + a], rbuf[a * KB + c]);
                vbuf[tt * KB + c] = acc;
            }
            __syncthreads();
            if (act) {
                T u[TR][4], v[4][4];
#pragma unroll
                for (int i = 0; i < TR; i++) vld<T, 4>(u[i], cbuf + row(i) * 4);
#pragma unroll
                for (int t = 0; t < 4; t++) vld<T, 4>(v[t], vbuf + t * KB + col(0));
#pragma unroll
                for (int i = 0; i < TR; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) {
                        T acc = s[i][jj];
#pragma unroll
                        for (int t = 0; t < 4; t++) acc = msub(acc, u[i][t], v[t][jj]);
                        s[i][jj] = acc;
                    }
            }
        }
        // columns of the inverse back by the diagonal: S^{-1} = (D^{-1} S)^{-1} D^{-1}
        if (act) {
            T dc[4];
            vld<T, 4>(dc, dg + col(0));
#pragma unroll
            for (int jj = 0; jj < 4; jj++) {
                const T rc = sc_rcp_fast(dc[jj]);
#pragma unroll
                for (int i = 0; i < TR; i++) s[i][jj] = s[i][jj] * rc;
            }
        }
        __syncthreads();
        return __syncthreads_and(ok ? 1 : 0) != 0;
    }

    __device__ __forceinline__ bool inverse_r1(Reg &s, T *buf) const
    {
        bool ok = true;
        for (int j = 0; j < KB; j++) {
            T *rb = buf + (j & 1) * 2 * KB; // row j
            T *cb = rb + KB;                // column j
            const int jr = j / TR, ir = j - jr * TR; // owner row group / slot
            const int jc = j / TC, ic = j - jc * TC; // owner column group / slot
            if (act) {
                if (ty == jr) {
                    T v[TC];
#pragma unroll
                    for (int jj = 0; jj < TC; jj++) {
                        v[jj] = s[0][jj];
#pragma unroll
                        for (int i = 1; i < TR; i++) v[jj] = (i == ir) ? s[i][jj] : v[jj];
                    }
                    vst<T, TC>(rb + col(0), v);
                }
                if (tx == jc) {
                    T v[TR];
#pragma unroll
                    for (int i = 0; i < TR; i++) {
                        v[i] = s[i][0];
#pragma unroll
                        for (int jj = 1; jj < TC; jj++) v[i] = (jj == ic) ? s[i][jj] : v[i];
                    }
                    vst<T, TR>(cb + row(0), v);
                }
            }
            __syncthreads();
            if (act) {
                const T piv = cb[j];
                if (!sc_finite_nonzero(piv)) ok = false;
                const T pr = sc_frcp(piv);
                T bv[TC], av[TR];
                vld<T, TC>(bv, rb + col(0));
                vld<T, TR>(av, cb + row(0));
#pragma unroll
                for (int jj = 0; jj < TC; jj++) bv[jj] = bv[jj] * pr; // b[c] / p
#pragma unroll
                for (int i = 0; i < TR; i++)
#pragma unroll
                    for (int jj = 0; jj < TC; jj++) s[i][jj] = msub(s[i][jj], av[i], bv[jj]);
                if (ty == jr) { // row j <- b / p
#pragma unroll
                    for (int i = 0; i < TR; i++)
#pragma unroll
                        for (int jj = 0; jj < TC; jj++) s[i][jj] = (i == ir) ? bv[jj] : s[i][jj];
                }
                if (tx == jc) { // column j <- -a / p, pivot <- 1 / p
#pragma unroll
                    for (int i = 0; i < TR; i++) {
                        const T cv = (row(i) == j) ? pr : -(av[i] * pr);
#pragma unroll
                        for (int jj = 0; jj < TC; jj++) s[i][jj] = (jj == ic) ? cv : s[i][jj];
                    }
                }
            }
        }
        __syncthreads();
        return __syncthreads_and(ok ? 1 : 0) != 0;
    }
};

// Two-sided partition kernels (spike_twist.cu, and their right-hand-side
// sweeps in spike_apply.cu): three shared tiles per CTA, the tile inverse's
// scratch inside one of them, four CTAs per SM.
// Threads per CTA of the product-only kernels among them (the spikes' sweeps
// and back substitution): 128 for 64-row tiles gives every thread an 8 x 4
// sub-tile, i.e. 1.5 bytes of shared-memory operand traffic per FMA instead
// of 2.  The kernels with a tile inverse keep 4 x 4 sub-tiles: the inverse's
// barrier-separated steps want the larger CTA.
template <int KB> struct TwNT {
    static constexpr int value = KB == 64 ? 128 : NTOf<KB>::value;
};
template <class T, int KB> struct TwistFits {
    using TL = Tile<T, KB, NTOf<KB>::value>;
    static constexpr size_t smem = 3 * sizeof(T) * TL::ELEMS + 64;
    static constexpr bool ok = KB >= 16 && KB <= 64 && TL::INV_BUF <= TL::ELEMS && 4 * (smem + 1024) <= 228 * 1024;
};

// c ? a : b on two register values, in a form the compiler cannot turn into
// a select of addresses (which would move a register array to local memory)
__device__ __forceinline__ float reg_sel(bool c, float a, float b)
{
    float r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.s32 p, %3, 0;\n\tselp.f32 %0, %1, %2, p;\n\t}"
        : "=f"(r)
        : "f"(a), "f"(b), "r"((int)c));
    return r;
}

// ------------------------------------------------------------ 8 x 8 sub-tiles
// A 64 x 64 FP32 tile on 64 threads, each owning an 8 x 8 register sub-tile.
// Per k step of a product a thread reads 8 elements of each operand (four
// 16-byte shared loads, sixteen wavefronts per warp) for 64 FMAs: a warp's
// shared-memory wavefronts then match what the FMA pipe retires (an SM
// retires four warp FMAs per wavefront), where a 4 x 4 sub-tile issues two
// wavefronts per four FMAs and caps the FMA pipe at half.
//
// Thread (tx, ty), tx, ty in 0..7: rows ty*8 .. ty*8+7 (contiguous) and the
// columns of two 4-wide chunks, tx*4 .. tx*4+3 and 32 + tx*4 .. 32 + tx*4+3,
// so the eight lanes of a quarter-warp (one ty, tx = 0..7) read 128
// contiguous bytes of a right operand row (no bank conflict) and broadcast
// one 32-byte piece of the transposed left operand.  A warp holds four
// sub-tile rows (32 rows of the tile) and all 64 columns.
template <class T, int KB> struct Tile88 {
    static_assert(KB == 64, "8 x 8 sub-tiles on 64 threads: 64-row tiles");
    static constexpr int TX = 8, TY = 8, TC = 8, TR = 8;
    static constexpr int HALF = KB / 2; // column offset of the second chunk
    static constexpr int LD = TileLD<T, KB>::value;
    static constexpr int ELEMS = KB * LD;
    static constexpr int ACTIVE = 64;
    static constexpr int NT = 64;
    static constexpr int INV_HALF = 12 * KB + 16;
    static constexpr int INV_BUF = 2 * INV_HALF + KB;

    using Reg = T[TR][TC];

    int tx, ty;
    int wr0, wr1, wc0, wc1;
    bool act;
    __device__ __forceinline__ Tile88(int tid)
    {
        const int warp = tid >> 5, lane = tid & 31;
        act = tid < ACTIVE;
        tx = lane & 7;
        ty = warp * 4 + (lane >> 3);
        wr0 = warp * 32;
        wr1 = wr0 + 32;
        wc0 = 0;
        wc1 = KB;
    }
    __device__ __forceinline__ int row(int i) const { return ty * TR + i; }
    __device__ __forceinline__ int col(int j) const { return (j >> 2) * HALF + tx * 4 + (j & 3); }

    // the eight entries of sub-tile row i <-> two 4-wide chunks of a row at p (p = row start)
    __device__ __forceinline__ void ld_row(T (&d)[TC], const T *p) const
    {
        T a[4], b[4];
        vld<T, 4>(a, p + tx * 4);
        vld<T, 4>(b, p + HALF + tx * 4);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            d[j] = a[j];
            d[4 + j] = b[j];
        }
    }
    __device__ __forceinline__ void st_row(T *p, const T (&d)[TC]) const
    {
        T a[4], b[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            a[j] = d[j];
            b[j] = d[4 + j];
        }
        vst<T, 4>(p + tx * 4, a);
        vst<T, 4>(p + HALF + tx * 4, b);
    }

    __device__ __forceinline__ void rzero(Reg &a) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) a[i][j] = sc_zero<T>();
    }
    __device__ __forceinline__ void rload(Reg &a, const T *s) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) ld_row(a[i], s + row(i) * LD);
    }
    __device__ __forceinline__ void rstore(T *s, const Reg &a) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) st_row(s + row(i) * LD, a[i]);
    }
    // shared tile, transposed (element (r, c) at c*LD + r)
    __device__ __forceinline__ void rstore_t(T *s, const Reg &a) const
    {
#pragma unroll
        for (int j = 0; j < TC; j++) {
            T c[TR];
#pragma unroll
            for (int i = 0; i < TR; i++) c[i] = a[i][j];
            vst<T, TR>(s + col(j) * LD + row(0), c);
        }
    }
    __device__ __forceinline__ void gload(Reg &a, const T *g) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) ld_row(a[i], g + row(i) * KB);
    }
    __device__ __forceinline__ void gstore(T *g, const Reg &a) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) st_row(g + row(i) * KB, a[i]);
    }
    __device__ __forceinline__ void gstore_t(T *g, const Reg &a) const
    {
#pragma unroll
        for (int j = 0; j < TC; j++) {
            T c[TR];
#pragma unroll
            for (int i = 0; i < TR; i++) c[i] = a[i][j];
            vst<T, TR>(g + col(j) * KB + row(0), c);
        }
    }
    // acc (+|-)= A B, A given transposed (At, column-major).  TRI as Tile::mm_tA:
    // 1 / 2 = A upper / lower triangular (a warp skips the k where its rows of
    // A are zero); 3 / 4 = B lower / upper triangular (a warp holds every
    // column, so nothing is skipped).  LDA / LDB: row strides of the operands
    // (LD padded, KB dense).
    template <bool SUB, int TRI = 0, int LDA = LD, int LDB = LD>
    __device__ __forceinline__ void mm_tA(Reg &acc, const T *At, const T *B) const
    {
        const int k0 = TRI == 1 ? wr0 : 0;
        const int k1 = TRI == 2 ? wr1 : KB;
#pragma unroll 2
        for (int k = k0; k < k1; k++) {
            T a[TR], b[TC];
            vld<T, TR>(a, At + k * LDA + row(0));
            ld_row(b, B + k * LDB);
#pragma unroll
            for (int i = 0; i < TR; i++)
#pragma unroll
                for (int j = 0; j < TC; j++) acc[i][j] = SUB ? msub(acc[i][j], a[i], b[j]) : madd(acc[i][j], a[i], b[j]);
        }
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mma_t(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<false, 0, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mms_t(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 0, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mma_tu(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<false, 1, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mms_tl(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 2, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mma_tl(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<false, 2, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD> __device__ __forceinline__ void mms_tu(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 1, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD>
    __device__ __forceinline__ void mms_t_bl(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 3, LDA, LDB>(acc, At, B);
    }
    template <int LDA = LD, int LDB = LD>
    __device__ __forceinline__ void mms_t_bu(Reg &acc, const T *At, const T *B) const
    {
        mm_tA<true, 4, LDA, LDB>(acc, At, B);
    }

    // In-place Gauss-Jordan inverse without pivoting, blocked by 4 x 4 pivot
    // blocks: the update of Tile::inverse_b4 (S <- S - U'V', U' = pivot
    // columns - I on the pivot rows, V' = P^{-1} (pivot rows + I on the pivot
    // columns)) on this layout.  Pivot block q covers rows and columns
    // 4q .. 4q+3: its rows are register rows 4 (q & 1) .. +3 of sub-tile row
    // q / 2, its columns register columns 4 (q / 8) .. +3 of sub-tile column
    // q & 7.  Rows are scaled to a unit diagonal first and the inverse's
    // columns back after.  buf: INV_BUF elements of shared memory (16-byte
    // aligned).  All threads must call; false in every thread on a zero or
    // non-finite pivot.  The register offsets of each step are template
    // arguments, so the sub-tile never leaves the registers.
    __device__ __forceinline__ bool inverse(Reg &s, T *buf) const
    {
        bool ok = true;
        T *dg = buf + 2 * INV_HALF; // the diagonal, KB entries
        // diagonal entry (c, c), c = h*32 + tx*4 + j, sits in sub-tile row
        // 4h + tx/2, register row 4 (tx & 1) + j, register column 4h + j
        const bool odd = (tx & 1) != 0;
#pragma unroll
        for (int h = 0; h < 2; h++)
            if (ty == 4 * h + (tx >> 1)) {
                T d[4];
#pragma unroll
                for (int j = 0; j < 4; j++) d[j] = reg_sel(odd, s[4 + j][4 * h + j], s[j][4 * h + j]);
                vst<T, 4>(dg + h * HALF + tx * 4, d);
            }
        __syncthreads();
        {
            T dr[TR];
            vld<T, TR>(dr, dg + row(0));
#pragma unroll
            for (int i = 0; i < TR; i++) {
                if (!sc_finite_nonzero(dr[i])) ok = false;
                const T rr = sc_rcp_fast(dr[i]);
#pragma unroll
                for (int jj = 0; jj < TC; jj++) s[i][jj] = s[i][jj] * rr;
            }
        }
        // q = 2 q2 + HQ; pivot columns in register columns 4..7 from q = 8 on
        for (int q2 = 0; q2 < KB / 16; q2++) {
            inv_step<false, 0>(s, buf, q2, ok);
            inv_step<false, 1>(s, buf, q2, ok);
        }
        for (int q2 = KB / 16; q2 < KB / 8; q2++) {
            inv_step<true, 0>(s, buf, q2, ok);
            inv_step<true, 1>(s, buf, q2, ok);
        }
        // columns of the inverse back by the diagonal: S^{-1} = (D^{-1} S)^{-1} D^{-1}
        {
            T dc[TC];
            ld_row(dc, dg);
#pragma unroll
            for (int jj = 0; jj < TC; jj++) {
                const T rc = sc_rcp_fast(dc[jj]);
#pragma unroll
                for (int i = 0; i < TR; i++) s[i][jj] = s[i][jj] * rc;
            }
        }
        __syncthreads();
        return __syncthreads_and(ok ? 1 : 0) != 0;
    }

    // one 4 x 4 pivot block of inverse(): q = 2 q2 + HQ, its rows register
    // rows 4 HQ .. 4 HQ + 3 of sub-tile row q2, its columns register columns
    // (HI ? 4 : 0) .. +3 of sub-tile column q & 7.  The eight owners of the
    // pivot rows are one quarter-warp: each takes the pivot block P from its
    // owner by shuffles, inverts it (the same steps in all eight, no barrier)
    // and forms its own columns of V' = P^{-1} (pivot rows + I); the owners of
    // the pivot columns publish U'.  One barrier, then every thread applies
    // S <- S - U' V' to its sub-tile.
    template <bool HI, int HQ> __device__ __forceinline__ void inv_step(Reg &s, T *buf, int q2, bool &ok) const
    {
        constexpr int CO = HI ? 4 : 0, RO = 4 * HQ;
        const int q = 2 * q2 + HQ;
        T *cbuf = buf + HQ * INV_HALF; // [KB][4] pivot columns U'
        T *vbuf = cbuf + 4 * KB;       // [4][KB] V'
        const bool rown = ty == q2, cown = tx == (q & 7);
        if (rown) {
            const int lane = threadIdx.x & 31;
            const unsigned qmask = 0xffu << (lane & 24);
            const int src = (lane & 24) + (q & 7); // the pivot block's owner in this quarter-warp
            T pinv[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) pinv[a][b] = __shfl_sync(qmask, s[RO + a][CO + b], src);
#pragma unroll
            for (int k = 0; k < 4; k++) { // unblocked Gauss-Jordan in registers
                const T piv = pinv[k][k];
                if (!sc_finite_nonzero(piv)) ok = false;
                const T pr = sc_rcp_fast(piv);
#pragma unroll
                for (int b = 0; b < 4; b++)
                    if (b != k) pinv[k][b] = pinv[k][b] * pr;
#pragma unroll
                for (int a = 0; a < 4; a++)
                    if (a != k) {
                        const T f = pinv[a][k];
#pragma unroll
                        for (int b = 0; b < 4; b++)
                            if (b != k) pinv[a][b] = msub(pinv[a][b], f, pinv[k][b]);
                        pinv[a][k] = -(f * pr);
                    }
                pinv[k][k] = pr;
            }
#pragma unroll
            for (int tt = 0; tt < 4; tt++) {
                T vrow[TC];
#pragma unroll
                for (int jj = 0; jj < TC; jj++) {
                    T acc = sc_zero<T>();
#pragma unroll
                    for (int a = 0; a < 4; a++) {
                        const T bb = (cown && jj == CO + a) ? s[RO + a][jj] + sc_one<T>() : s[RO + a][jj];
                        acc = madd(acc, pinv[tt][a], bb);
                    }
                    vrow[jj] = acc;
                }
                st_row(vbuf + tt * KB, vrow);
            }
        }
        if (cown) {
#pragma unroll
            for (int i = 0; i < TR; i++) {
                T u[4];
#pragma unroll
                for (int t = 0; t < 4; t++) u[t] = (rown && i == RO + t) ? s[i][CO + t] - sc_one<T>() : s[i][CO + t];
                vst<T, 4>(cbuf + row(i) * 4, u);
            }
        }
        __syncthreads();
        T u[TR][4], v[4][TC];
#pragma unroll
        for (int i = 0; i < TR; i++) vld<T, 4>(u[i], cbuf + row(i) * 4);
#pragma unroll
        for (int t = 0; t < 4; t++) ld_row(v[t], vbuf + t * KB);
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int jj = 0; jj < TC; jj++) {
                T acc = s[i][jj];
#pragma unroll
                for (int t = 0; t < 4; t++) acc = msub(acc, u[i][t], v[t][jj]);
                s[i][jj] = acc;
            }
    }
};

// ------------------------------------------------------------ one warp per tile
// A KB x KB FP32 tile (KB = 16 or 32) on ONE warp, each lane owning a
// KB/8 x KB/4 register sub-tile: lane (a, b), a = lane / 4, b = lane % 4,
// holds rows a KB/8 .. a KB/8 + KB/8 - 1 and columns b KB/4 .. b KB/4 +
// KB/4 - 1 (4 x 8 at KB = 32).  A chain on one warp needs no CTA barrier:
// the tile inverse runs on shuffles alone (pivot rows and columns travel
// between lanes).  Per k step of a product a lane reads KB/8 elements of the
// transposed left operand and KB/4 of the right operand in 8- or 16-byte
// pieces for KB^2/32 FMAs, so FMAs are most of what it issues; for tiles this
// small many chains share each SM, and the instructions per FMA are what
// bound them.  Shared tiles are dense (row stride KB): they arrive by single
// bulk copies.
template <class T, int KB> struct TileW {
    static_assert((KB == 16 || KB == 32) && sizeof(T) == 4, "one warp per 16- or 32-row FP32 tile");
    static constexpr int TR = KB / 8, TC = KB / 4;
    static constexpr int LD = KB;
    static constexpr int ELEMS = KB * KB;
    static constexpr int NT = 32;
    static constexpr bool act = true; // every lane holds part of the tile

    using Reg = T[TR][TC];

    int a, b;
    __device__ __forceinline__ TileW(int lane)
    {
        a = (lane & 31) >> 2;
        b = lane & 3;
    }
    __device__ __forceinline__ int row(int i) const { return a * TR + i; }
    __device__ __forceinline__ int col(int j) const { return b * TC + j; }

    __device__ __forceinline__ void ld_row(T (&d)[TC], const T *p) const { vld<T, TC>(d, p + b * TC); }
    __device__ __forceinline__ void st_row(T *p, const T (&d)[TC]) const { vst<T, TC>(p + b * TC, d); }
    __device__ __forceinline__ void rzero(Reg &x) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) x[i][j] = sc_zero<T>();
    }
    // dense tile (shared or global, row stride KB), row-major, and transposed
    // (element (r, c) at c * KB + r)
    __device__ __forceinline__ void rload(Reg &x, const T *s) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) ld_row(x[i], s + row(i) * LD);
    }
    __device__ __forceinline__ void rstore(T *s, const Reg &x) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) st_row(s + row(i) * LD, x[i]);
    }
    __device__ __forceinline__ void rstore_t(T *s, const Reg &x) const
    {
#pragma unroll
        for (int j = 0; j < TC; j++) {
            T c[TR];
#pragma unroll
            for (int i = 0; i < TR; i++) c[i] = x[i][j];
            vst<T, TR>(s + col(j) * LD + row(0), c);
        }
    }
    __device__ __forceinline__ void gload(Reg &x, const T *g) const { rload(x, g); }
    __device__ __forceinline__ void gstore(T *g, const Reg &x) const { rstore(g, x); }
    __device__ __forceinline__ void gstore_t(T *g, const Reg &x) const { rstore_t(g, x); }
    // acc += D (a dense row-major tile)
    __device__ __forceinline__ void radd(Reg &acc, const T *s) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++) {
            T d[TC];
            ld_row(d, s + row(i) * LD);
#pragma unroll
            for (int j = 0; j < TC; j++) acc[i][j] = acc[i][j] + d[j];
        }
    }
    // acc (+|-)= A B, A given transposed (At, column-major), both dense
    template <bool SUB> __device__ __forceinline__ void mm_tA(Reg &acc, const T *At, const T *B) const
    {
#pragma unroll 4
        for (int k = 0; k < KB; k++) {
            T x[TR], y[TC];
            vld<T, TR>(x, At + k * LD + row(0));
            ld_row(y, B + k * LD);
#pragma unroll
            for (int i = 0; i < TR; i++)
#pragma unroll
                for (int j = 0; j < TC; j++) acc[i][j] = SUB ? msub(acc[i][j], x[i], y[j]) : madd(acc[i][j], x[i], y[j]);
        }
    }

    // In-place Gauss-Jordan inverse without pivoting, one pivot at a time, on
    // shuffles: pivot k's row lives in lanes (k / TR, *), register row k % TR;
    // its column in lanes (*, k / TC), register column k % TC.  Each pivot
    // applies S <- S - u v' with u = (pivot column) - e_k and
    // v = ((pivot row) + e_k) / S(k, k), which leaves S(k, k) = 1 / S(k, k),
    // the pivot row scaled and the pivot column negated and scaled, as
    // Gauss-Jordan does.  Rows are scaled to a unit diagonal first and the
    // inverse's columns back after (S^{-1} = (D^{-1} S)^{-1} D^{-1}), as the
    // CTA tiles' inverses do.  false in every lane on a zero or non-finite
    // pivot or diagonal entry.
    __device__ __forceinline__ bool inverse(Reg &s) const
    {
        constexpr unsigned FULL = 0xffffffffu;
        bool ok = true;
        // diagonal entry (TR a + i, TR a + i) sits in lane (a, a / 2),
        // register [i][TR (a & 1) + i]
        T dr[TR];
        const bool odd = (a & 1) != 0;
        const int dsrc = (a << 2) | (a >> 1);
#pragma unroll
        for (int i = 0; i < TR; i++) dr[i] = __shfl_sync(FULL, reg_sel(odd, s[i][TR + i], s[i][i]), dsrc);
#pragma unroll
        for (int i = 0; i < TR; i++) {
            if (!sc_finite_nonzero(dr[i])) ok = false;
            const T rr = sc_rcp_fast(dr[i]);
#pragma unroll
            for (int j = 0; j < TC; j++) s[i][j] = s[i][j] * rr;
        }
        for (int kb = 0; kb < KB / TC; kb++) { // TC pivots per pass: those of column group kb
#pragma unroll
            for (int kk = 0; kk < TC; kk++) {
                const int ra = 2 * kb + kk / TR; // owner row group of pivot k = TC kb + kk
                T prow[TC], pcol[TR];
#pragma unroll
                for (int j = 0; j < TC; j++) prow[j] = __shfl_sync(FULL, s[kk % TR][j], (ra << 2) | b);
#pragma unroll
                for (int i = 0; i < TR; i++) pcol[i] = __shfl_sync(FULL, s[i][kk], (a << 2) | kb);
                const T piv = __shfl_sync(FULL, s[kk % TR][kk], (ra << 2) | kb);
                if (!sc_finite_nonzero(piv)) ok = false;
                const T pinv = sc_rcp_fast(piv);
                const bool mycol = b == kb, myrow = a == ra;
                T v[TC];
#pragma unroll
                for (int j = 0; j < TC; j++)
                    v[j] = (j == kk ? prow[j] + (mycol ? sc_one<T>() : sc_zero<T>()) : prow[j]) * pinv;
#pragma unroll
                for (int i = 0; i < TR; i++) {
                    const T u = i == kk % TR ? pcol[i] - (myrow ? sc_one<T>() : sc_zero<T>()) : pcol[i];
#pragma unroll
                    for (int j = 0; j < TC; j++) s[i][j] = msub(s[i][j], u, v[j]);
                }
            }
        }
        // columns back by the diagonal: column TC b + j's entry of dr sits in
        // lane (2b + j / TR, *), register j % TR
#pragma unroll
        for (int j = 0; j < TC; j++) {
            const T dc = __shfl_sync(FULL, dr[j % TR], ((2 * b + j / TR) << 2) | b);
            const T rc = sc_rcp_fast(dc);
#pragma unroll
            for (int i = 0; i < TR; i++) s[i][j] = s[i][j] * rc;
        }
        return __all_sync(FULL, ok) != 0;
    }
};

// Thread counts and tile geometry of the two-sided kernels: the elimination
// chains of FP32 64-row tiles run on 64 threads with 8 x 8 sub-tiles (Tile88),
// everything else on the Tile layouts above (NTOf threads for the kernels with
// a tile inverse, TwNT for the product-only ones, whose 8 x 4 sub-tiles on 128
// threads timed faster than 8 x 8 on 64: more warps hide the loads).
template <class T, int KB> struct TwCfg {
    static constexpr bool T88 = sizeof(T) == 4 && KB == 64 && TileLD<T, KB>::value == KB + 4;
    static constexpr int NT_LU = T88 ? 64 : NTOf<KB>::value;
    static constexpr int NT_PROD = TwNT<KB>::value;
};
template <class T, int KB, bool T88 = TwCfg<T, KB>::T88> struct TwTiles {
    using LU = Tile<T, KB, TwCfg<T, KB>::NT_LU>;
    using PROD = Tile<T, KB, TwCfg<T, KB>::NT_PROD>;
};
template <class T, int KB> struct TwTiles<T, KB, true> {
    using LU = Tile88<T, KB>;
    using PROD = Tile<T, KB, TwCfg<T, KB>::NT_PROD>;
};

// Dense global tile (KB*KB elements, 16-byte aligned) -> shared tile with row
// stride TileLD (the element order is kept: a column-major global tile lands
// as a transposed shared tile).  Every thread issues all of its 16-byte loads
// before its first shared-memory store, so a tile costs one memory round trip.
template <class T, int KB, int NT> __device__ __forceinline__ void copy_tile_g2s(T *s, const T *g)
{
    constexpr int EPC = 16 / sizeof(T) > 0 ? 16 / sizeof(T) : 1; // elements per 16-byte chunk
    constexpr int CH = KB * KB / EPC;                             // chunks per tile
    constexpr int PER = (CH + NT - 1) / NT;                       // chunks per thread
    const uint4 *src = reinterpret_cast<const uint4 *>(g);
    uint4 buf[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int c = threadIdx.x + i * NT;
        if (c < CH) buf[i] = __ldg(src + c);
    }
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int c = threadIdx.x + i * NT;
        if (c < CH) {
            const T *e = reinterpret_cast<const T *>(&buf[i]);
#pragma unroll
            for (int k = 0; k < EPC; k++) {
                const int q = c * EPC + k, r = q / KB, cc = q - r * KB;
                s[r * TileLD<T, KB>::value + cc] = e[k];
            }
        }
    }
}

// ------------------------------------------------------------ async copies
// cp.async (global -> shared, 16 bytes, bypassing registers and L1); used to
// fetch the next block's tiles while the current block computes.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
// all but the N most recently committed groups complete
template <int N> __device__ __forceinline__ void cp_async_wait_n()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
// 8- and 4-byte asynchronous copies (both addresses aligned to the size)
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
// one element of E bytes (4, 8 or 16, naturally aligned)
template <int E> __device__ __forceinline__ void cp_async_elem(void *smem, const void *gmem)
{
    if constexpr (E == 16)
        cp_async16(smem, gmem);
    else if constexpr (E == 8)
        cp_async8(smem, gmem);
    else
        cp_async4(smem, gmem);
}
// ------------------------------------------------------------ bulk copies (TMA) with mbarriers
// A tile lands in shared memory by one bulk copy per row
// (cp.async.bulk global -> shared, issued by one warp), each completing its
// bytes on the tile's mbarrier; the threads that read the tile wait on the
// barrier's phase.  Rows are KB * sizeof(T) >= 64 bytes and the shared rows
// keep their 16-byte padding (TileLD), so both ends stay 16-byte aligned and
// the padded layout (no bank conflicts) is unchanged.  The copies read this
// GPU's own memory into the issuing CTA's shared memory only (no cluster, no
// multicast).
// A wait on a bulk copy gives up after SPK_MBAR_TIMEOUT_NS of the GPU's global
// timer (or SPK_MBAR_SPIN_LIMIT polls, whichever comes first); each poll
// suspends the thread for at most SPK_MBAR_POLL_NS unless the phase completes.
#define SPK_MBAR_TIMEOUT_NS 1000000000ull /* 1 s */
#define SPK_MBAR_POLL_NS 20000u           /* 20 us */
#define SPK_MBAR_SPIN_LIMIT (1 << 24)

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// make the initialised barriers visible to the copy engine's proxy
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// order this thread's earlier generic-proxy shared accesses before later bulk copies into them
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// true when the phase with parity `parity` has completed; otherwise the thread
// may be suspended for up to SPK_MBAR_POLL_NS (woken early when the phase
// completes) before false comes back
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_u32(bar)), "r"(parity), "r"(SPK_MBAR_POLL_NS)
                 : "memory");
    return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase of `bar` with parity `parity` to complete.  Gives up --
// returns false -- after SPK_MBAR_TIMEOUT_NS on the global timer (or
// SPK_MBAR_SPIN_LIMIT polls), so a copy that never lands ends in an error
// status instead of a hang.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (int i = 0; i < SPK_MBAR_SPIN_LIMIT; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > SPK_MBAR_TIMEOUT_NS) break;
    }
    return false;
}
// Dense global tile (KB x KB, row-major or column-major as stored) -> shared
// tile with row stride TileLD, by KB bulk copies on `bar`.  Called by all 32
// lanes of one warp, after a barrier that ends every read of `s`.
template <class T, int KB> __device__ __forceinline__ void bulk_tile(T *s, const T *g, uint64_t *bar)
{
    constexpr int LD = TileLD<T, KB>::value;
    constexpr unsigned ROW = KB * sizeof(T);
    static_assert(ROW % 16 == 0 && (LD * sizeof(T)) % 16 == 0, "bulk copies move 16-byte multiples");
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, ROW * KB);
    }
    __syncwarp();
    for (int r = lane; r < KB; r += 32) bulk_g2s(s + r * LD, g + (size_t)r * KB, ROW, bar);
}
// Dense global tile -> dense shared tile (row stride KB): one bulk copy of
// KB * KB elements.  For tiles that serve only as operands read in whole
// 16-byte pieces -- the transposed left operand, whose lanes broadcast, or a
// right operand read in contiguous runs -- where the padding buys nothing and
// one copy replaces KB row copies.  Called by all 32 lanes of one warp, after
// a barrier that ends every read of `s`.
template <class T, int KB> __device__ __forceinline__ void bulk_tile_dense(T *s, const T *g, uint64_t *bar)
{
    constexpr unsigned BYTES = KB * KB * sizeof(T);
    static_assert(BYTES % 16 == 0, "bulk copies move 16-byte multiples");
    if ((threadIdx.x & 31) == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, BYTES);
        bulk_g2s(s, g, BYTES, bar);
    }
}

// One shared tile's barrier as every thread of the CTA tracks it: the parity
// of its next phase and whether a copy is in flight.  All threads call
// issue() / issue_dense() (warp 0 issues the copies) and wait(), on uniform
// conditions.
struct TileBar {
    uint64_t *bar;
    unsigned phase;
    bool inflight;
    template <class T, int KB> __device__ __forceinline__ void issue(T *s, const T *g)
    {
        if (threadIdx.x < 32) bulk_tile<T, KB>(s, g, bar);
        inflight = true;
    }
    template <class T, int KB> __device__ __forceinline__ void issue_dense(T *s, const T *g)
    {
        if (threadIdx.x < 32) bulk_tile_dense<T, KB>(s, g, bar);
        inflight = true;
    }
    // wait for the tile in flight; false on a timeout
    __device__ __forceinline__ bool wait()
    {
        const bool ok = mbar_wait(bar, phase);
        phase ^= 1u;
        inflight = false;
        return ok;
    }
    // before leaving the kernel: let a copy still in flight land (bounded)
    __device__ __forceinline__ void drain()
    {
        if (inflight) wait();
    }
};

// ------------------------------------------------------------ tile rows across lanes
// A chain of a small band (KB <= 4) runs on KB consecutive lanes of a warp:
// lane r owns row r of every KB x KB tile, and rows of another lane arrive by
// shuffles within the KB-lane segment (mask: the segment's lanes only).
template <int KB> __device__ __forceinline__ unsigned seg_mask()
{
    const unsigned lane = threadIdx.x & 31u;
    return (KB == 32 ? 0xffffffffu : ((1u << KB) - 1u)) << (lane & ~(unsigned)(KB - 1));
}
template <int KB> __device__ __forceinline__ float seg_shfl(unsigned m, float v, int src)
{
    return __shfl_sync(m, v, src, KB);
}
template <int KB> __device__ __forceinline__ double seg_shfl(unsigned m, double v, int src)
{
    return __shfl_sync(m, v, src, KB);
}
template <int KB> __device__ __forceinline__ cfloat seg_shfl(unsigned m, cfloat v, int src)
{
    return {__shfl_sync(m, v.re, src, KB), __shfl_sync(m, v.im, src, KB)};
}
template <int KB> __device__ __forceinline__ cdouble seg_shfl(unsigned m, cdouble v, int src)
{
    return {__shfl_sync(m, v.re, src, KB), __shfl_sync(m, v.im, src, KB)};
}
// out = this lane's row of A B, a: the lane's row of A, b: the lane's row of B
template <class T, int KB>
__device__ __forceinline__ void row_mul(unsigned m, T (&out)[KB], const T (&a)[KB], const T (&b)[KB])
{
#pragma unroll
    for (int c = 0; c < KB; c++) out[c] = sc_zero<T>();
#pragma unroll
    for (int k = 0; k < KB; k++)
#pragma unroll
        for (int c = 0; c < KB; c++) out[c] = madd(out[c], a[k], seg_shfl<KB>(m, b[c], k));
}
// out -= this lane's row of A B
template <class T, int KB>
__device__ __forceinline__ void row_msub(unsigned m, T (&out)[KB], const T (&a)[KB], const T (&b)[KB])
{
#pragma unroll
    for (int k = 0; k < KB; k++)
#pragma unroll
        for (int c = 0; c < KB; c++) out[c] = msub(out[c], a[k], seg_shfl<KB>(m, b[c], k));
}
// In-place Gauss-Jordan inverse without pivoting of the tile whose row r this
// lane holds, pivot rows broadcast by shuffle (S[j][c] *= 1/p, S[j][j] = 1/p;
// S[r][c] -= S[r][j] S[j][c], S[r][j] = -S[r][j]/p).  false on a zero or
// non-finite pivot (in every lane).
template <class T, int KB> __device__ __forceinline__ bool row_inv(unsigned m, T (&s)[KB], int r)
{
    bool ok = true;
#pragma unroll
    for (int j = 0; j < KB; j++) {
        const T piv = seg_shfl<KB>(m, s[j], j);
        if (!sc_finite_nonzero(piv)) ok = false;
        const T ip = sc_rcp_fast(piv);
        if (r == j) {
#pragma unroll
            for (int c = 0; c < KB; c++)
                if (c != j) s[c] = s[c] * ip;
            s[j] = ip;
        }
        T pr[KB];
#pragma unroll
        for (int c = 0; c < KB; c++) pr[c] = seg_shfl<KB>(m, s[c], j);
        if (r != j) {
            const T a = s[j];
#pragma unroll
            for (int c = 0; c < KB; c++)
                if (c != j) s[c] = msub(s[c], a, pr[c]);
            s[j] = -(a * ip);
        }
    }
    return ok;
}

// ------------------------------------------------------------ tiles on lanes, one element each
// A chain of a tiny band (KB <= 4) that is mostly products and inverses runs
// on KB*KB consecutive lanes: lane e of the segment holds element (e / KB,
// e % KB) of every KB x KB tile, so a tile product is KB pairs of shuffles and
// one multiply-add per lane (a lane holding a whole row needs KB times that).
// out(r, c) = sum_k A(r, k) B(k, c)
template <class T, int KB> __device__ __forceinline__ T el_mul(unsigned m, T a, T b, int r, int c)
{
    constexpr int EL = KB * KB;
    T acc = sc_zero<T>();
#pragma unroll
    for (int k = 0; k < KB; k++) acc = madd(acc, seg_shfl<EL>(m, a, r * KB + k), seg_shfl<EL>(m, b, k * KB + c));
    return acc;
}
// out(r, c) - sum_k A(r, k) B(k, c)
template <class T, int KB> __device__ __forceinline__ T el_msub(unsigned m, T out, T a, T b, int r, int c)
{
    constexpr int EL = KB * KB;
#pragma unroll
    for (int k = 0; k < KB; k++) out = msub(out, seg_shfl<EL>(m, a, r * KB + k), seg_shfl<EL>(m, b, k * KB + c));
    return out;
}
// In-place Gauss-Jordan inverse without pivoting, the same steps as row_inv
// on elements: S[j][c] *= 1/p, S[j][j] = 1/p; S[r][c] -= S[r][j] S[j][c],
// S[r][j] = -S[r][j]/p.  false on a zero or non-finite pivot (in every lane).
template <class T, int KB> __device__ __forceinline__ bool el_inv(unsigned m, T &s, int r, int c)
{
    constexpr int EL = KB * KB;
    bool ok = true;
#pragma unroll
    for (int j = 0; j < KB; j++) {
        const T piv = seg_shfl<EL>(m, s, j * KB + j);
        if (!sc_finite_nonzero(piv)) ok = false;
        const T ip = sc_rcp_fast(piv);
        if (r == j) s = c == j ? ip : s * ip;
        const T rowj = seg_shfl<EL>(m, s, j * KB + c); // S[j][c], scaled
        const T colj = seg_shfl<EL>(m, s, r * KB + j); // S[r][j] (unchanged so far for r != j)
        if (r != j) s = c == j ? -(colj * ip) : msub(s, colj, rowj);
    }
    return ok;
}

// Chains per CTA at launch: spread the chains over every SM (two CTAs each
// where there are enough), at most cpc_max per CTA.
static inline int chains_per_cta(long long chains, int cpc_max)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    long long c = (chains + 2LL * sms - 1) / (2LL * sms);
    if (c < 1) c = 1;
    if (c > cpc_max) c = cpc_max;
    return (int)c;
}

// threads per CTA of a chain kernel whose threads each stage `bytes` in shared memory
__host__ __device__ constexpr int chain_threads(int bytes)
{
    return (98304 / bytes) >= 128 ? 128 : (98304 / bytes) >= 64 ? 64 : 32;
}

// Dense global tile -> shared tile (row stride TileLD), asynchronously.  Tiles
// whose rows are shorter than 16 bytes (FP32 with KB = 2) are copied
// synchronously instead.  The caller commits, waits and synchronizes.
template <class T, int KB, int NT> __device__ __forceinline__ void cp_async_tile(T *s, const T *g)
{
    if constexpr (KB * sizeof(T) < 16) {
        copy_tile_g2s<T, KB, NT>(s, g);
    } else {
        constexpr int EPC = 16 / sizeof(T) > 0 ? 16 / sizeof(T) : 1;
        constexpr int CH = KB * KB / EPC;
        constexpr int LD = TileLD<T, KB>::value;
        for (int c = threadIdx.x; c < CH; c += NT) {
            const int q = c * EPC, r = q / KB, cc = q - r * KB;
            cp_async16(s + r * LD + cc, g + q);
        }
    }
}

// FP64 -> FP32, round to nearest even, with integer instructions: GB300's FP64
// pipe (which executes the F2F conversion) is ~60x narrower than its integer
// pipe.  Normal results only; zero, subnormal, overflow, inf and NaN take the
// hardware conversion.  Bit-identical to (float)x.
// The rare cases call out of line so the compiler keeps them a branch: an
// if-converted hardware conversion would run on the FP64 pipe for every value.
static __device__ __noinline__ float f64_to_f32_rare(double x) { return (float)x; }
static __device__ __noinline__ double f32_to_f64_rare(float x) { return (double)x; }
__device__ __forceinline__ float f64_to_f32(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 255) return f64_to_f32_rare(x);
    const unsigned r = ((hi & 0xfffffu) << 3) | (lo >> 29); // 23 mantissa bits
    const unsigned rem = lo & 0x1fffffffu;                  // 29 dropped bits
    const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (r & 1u));
    // a carry out of the mantissa bumps the exponent (to inf at the top), as it should
    return __uint_as_float(((hi & 0x80000000u) | ((unsigned)e << 23)) + r + up);
}
// FP32 -> FP64 (exact) with integer instructions, for the same reason.  Normal
// inputs only; zero, subnormal, inf and NaN take the hardware conversion.
__device__ __forceinline__ double f32_to_f64(float x)
{
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return f32_to_f64_rare(x);
    const unsigned hi = (u & 0x80000000u) | ((e + (1023u - 127u)) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}
template <class T, class H> __device__ __forceinline__ T cvt_fast(H v) { return sc_cvt<T, H>(v); }
template <> __device__ __forceinline__ double cvt_fast<double, float>(float v) { return f32_to_f64(v); }
template <> __device__ __forceinline__ cdouble cvt_fast<cdouble, cfloat>(cfloat v)
{
    return {f32_to_f64(v.re), f32_to_f64(v.im)};
}
template <> __device__ __forceinline__ float cvt_fast<float, double>(double v) { return f64_to_f32(v); }
template <> __device__ __forceinline__ cfloat cvt_fast<cfloat, cdouble>(cdouble v)
{
    return {f64_to_f32(v.re), f64_to_f32(v.im)};
}

// ------------------------------------------------------------ warp sums
// __shfl_xor_sync for any scalar (complex types move as 32-bit words)
template <class T> __device__ __forceinline__ T shfl_xor_any(T v, int off)
{
    if constexpr (sizeof(T) == 4) {
        return __shfl_xor_sync(0xffffffffu, v, off);
    } else {
        T other;
        const unsigned *src = (const unsigned *)&v;
        unsigned *dst = (unsigned *)&other;
#pragma unroll
        for (int w = 0; w < (int)(sizeof(T) / 4); w++) dst[w] = __shfl_xor_sync(0xffffffffu, src[w], off);
        return other;
    }
}

// Sums V per-lane values over each group of W consecutive lanes at once (V,
// W powers of two, V <= W <= 32): each exchange step halves the values a lane
// holds, so the whole reduction takes V - 1 + log2 W - log2 V shuffles instead
// of V log2 W.  Afterwards v[0] of lane l holds its group's total of value
// index (l mod W) >> (log2 W - log2 V).
template <int N, int OFF, class T, int V> __device__ __forceinline__ void warp_tsum_step(T (&v)[V], int lane)
{
    if constexpr (OFF >= 1) {
        if constexpr (N > 1) {
            constexpr int H = N / 2;
            const bool up = (lane & OFF) != 0;
#pragma unroll
            for (int j = 0; j < H; j++) {
                const T send = up ? v[j] : v[j + H];
                const T keep = up ? v[j + H] : v[j];
                v[j] = keep + shfl_xor_any(send, OFF);
            }
            warp_tsum_step<H, OFF / 2>(v, lane);
        } else {
            v[0] = v[0] + shfl_xor_any(v[0], OFF);
            warp_tsum_step<1, OFF / 2>(v, lane);
        }
    }
}
template <class T, int V, int W = 32> __device__ __forceinline__ T warp_tsum(T (&v)[V], int lane)
{
    static_assert(V >= 1 && V <= W && W <= 32 && (V & (V - 1)) == 0 && (W & (W - 1)) == 0,
                  "V <= W <= 32, powers of two");
    warp_tsum_step<V, W / 2>(v, lane);
    return v[0];
}

// 16-byte-aligned carve-up of dynamic shared memory
__device__ __forceinline__ char *smem_align(char *p)
{
    return (char *)(((uintptr_t)p + 15) & ~(uintptr_t)15);
}

#define SPK_CHECK_LAUNCH()                                                                      \
    do {                                                                                        \
        cudaError_t e_ = cudaGetLastError();                                                    \
        if (e_ != cudaSuccess) return SPK_ECUDA;                                                \
    } while (0)
