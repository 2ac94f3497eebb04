// spike_common.cuh -- scalar types and KB x KB tile operations shared by the
// SPIKE kernels (sm_103a).
//
// Every dense block of the block-tridiagonal view of A_i is a KB x KB tile.
// A CTA of NT threads owns one tile operation at a time; each active thread
// holds a TR x TC register sub-tile at rows ty + i*TY, columns tx + j*TX
// (strided so that a warp's shared-memory reads are conflict-free).  Shared
// memory tiles are row-major with stride LD = KB + 1.
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
    static constexpr int value = KB >= 64 ? 256 : KB == 32 ? 128 : KB == 16 ? 64 : 32;
};

// ------------------------------------------------------------ tile geometry
template <class T, int KB, int NT> struct Tile {
    static constexpr int TX = KB < 16 ? KB : 16;
    static constexpr int TY0 = NT / TX;
    static constexpr int TY = TY0 < KB ? TY0 : KB;
    static constexpr int TC = KB / TX;
    static constexpr int TR = KB / TY;
    static constexpr int LD = KB + 1;        // shared-memory row stride
    static constexpr int ELEMS = KB * LD;    // shared-memory tile size
    static constexpr int ACTIVE = TX * TY;   // threads that own a sub-tile

    using Reg = T[TR][TC];

    int tx, ty;
    bool act;
    __device__ Tile(int tid)
    {
        act = tid < ACTIVE;
        tx = tid % TX;
        ty = tid / TX;
    }
    __device__ int row(int i) const { return ty + i * TY; }
    __device__ int col(int j) const { return tx + j * TX; }

    __device__ void rzero(Reg &a) const
    {
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) a[i][j] = sc_zero<T>();
    }
    // register tile <- shared tile (threads without a sub-tile hold zeros and
    // never touch shared memory: their row() is past the tile)
    __device__ void rload(Reg &a, const T *s) const
    {
        if (!act) {
            rzero(a);
            return;
        }
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) a[i][j] = s[row(i) * LD + col(j)];
    }
    // shared tile <- register tile (alpha * a)
    __device__ void rstore(T *s, const Reg &a) const
    {
        if (!act) return;
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) s[row(i) * LD + col(j)] = a[i][j];
    }
    // dense global tile (row-major, ld KB) <- register tile
    __device__ void gstore(T *g, const Reg &a) const
    {
        if (!act) return;
#pragma unroll
        for (int i = 0; i < TR; i++)
#pragma unroll
            for (int j = 0; j < TC; j++) g[row(i) * KB + col(j)] = a[i][j];
    }
    // acc += A * B (A, B shared tiles)
    __device__ void mma(Reg &acc, const T *A, const T *B) const
    {
        if (!act) return;
#pragma unroll 4
        for (int k = 0; k < KB; k++) {
            T a[TR], b[TC];
#pragma unroll
            for (int i = 0; i < TR; i++) a[i] = A[row(i) * LD + k];
#pragma unroll
            for (int j = 0; j < TC; j++) b[j] = B[k * LD + col(j)];
#pragma unroll
            for (int i = 0; i < TR; i++)
#pragma unroll
                for (int j = 0; j < TC; j++) acc[i][j] = madd(acc[i][j], a[i], b[j]);
        }
    }
    // acc -= A * B
    __device__ void mms(Reg &acc, const T *A, const T *B) const
    {
        if (!act) return;
#pragma unroll 4
        for (int k = 0; k < KB; k++) {
            T a[TR], b[TC];
#pragma unroll
            for (int i = 0; i < TR; i++) a[i] = A[row(i) * LD + k];
#pragma unroll
            for (int j = 0; j < TC; j++) b[j] = B[k * LD + col(j)];
#pragma unroll
            for (int i = 0; i < TR; i++)
#pragma unroll
                for (int j = 0; j < TC; j++) acc[i][j] = msub(acc[i][j], a[i], b[j]);
        }
    }

    // In-place Gauss-Jordan inverse of the register tile, no pivoting (the
    // diagonal blocks of a diagonally dominant A stay diagonally dominant
    // under block elimination).  buf: 4*KB scratch elements of shared memory.
    // All NT threads must call.  Returns false in every thread if a pivot was
    // zero or not finite.
    __device__ bool inverse(Reg &s, T *buf) const
    {
        bool ok = true;
        for (int j = 0; j < KB; j++) {
            T *rb = buf + (j & 1) * 2 * KB;
            T *cb = rb + KB;
            if (act) {
                const int jr = j % TY, ir = j / TY;
                const int jc = j % TX, ic = j / TX;
                if (ty == jr) {
#pragma unroll
                    for (int i = 0; i < TR; i++)
                        if (i == ir)
#pragma unroll
                            for (int jj = 0; jj < TC; jj++) rb[col(jj)] = s[i][jj];
                }
                if (tx == jc) {
#pragma unroll
                    for (int jj = 0; jj < TC; jj++)
                        if (jj == ic)
#pragma unroll
                            for (int i = 0; i < TR; i++) cb[row(i)] = s[i][jj];
                }
            }
            __syncthreads();
            if (act) {
                T piv = rb[j];
                if (!sc_finite_nonzero(piv)) ok = false;
                T p = sc_recip(piv);
                T rp[TC];
#pragma unroll
                for (int jj = 0; jj < TC; jj++) rp[jj] = rb[col(jj)] * p;
#pragma unroll
                for (int i = 0; i < TR; i++) {
                    const int r = row(i);
                    const T f = cb[r];
#pragma unroll
                    for (int jj = 0; jj < TC; jj++) {
                        const int c = col(jj);
                        T v;
                        if (r == j)
                            v = (c == j) ? p : rp[jj];
                        else
                            v = (c == j) ? -(f * p) : msub(s[i][jj], f, rp[jj]);
                        s[i][jj] = v;
                    }
                }
            }
        }
        __syncthreads();
        return __syncthreads_and(ok ? 1 : 0) != 0;
    }
};

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
