// spike_twist.cu -- two-sided ("twisted") partition factorization on sm_103a.
//
// A partition of N row blocks is eliminated from both ends at once: blocks
// 0..M-1 top-down (block LU, the recurrences of k_factor_fwd), blocks
// N-1..M+1 bottom-up (block UL), and the two chains meet at block M = N/2,
// which takes the bottom chain's Schur complement in place of D_M:
//
//   top     L_J = A(J,J-1) G_{J-1},  S_J = D_J - L_J A(J-1,J),  G_J = S_J^{-1}
//   bottom  U_J = A(J,J+1) H_{J+1},  T_J = D_J - U_J A(J+1,J),  H_J = T_J^{-1}
//   middle  T'_M = D_M - U_M A(M+1,M),  L_M = A(M,M-1) G_{M-1},
//           G_M = (T'_M - L_M A(M-1,M))^{-1}
//
// A solve sweeps both halves towards block M and back out again, so every
// sequential chain is half as long and a partition keeps two CTAs busy.  The
// arithmetic per block is the same as the one-sided factorization; the
// reference factors each A_i with SuperLU (OpenMP/spike_superlu.c:763) and
// solves its spikes column by column (OpenMP/spike_interfaces.c:143-209).
// These kernels hold three tiles in shared memory (the tile inverse borrows
// whichever one is idle) so that four CTAs share an SM; the one-sided kernels
// hold six.
//
//   k_tw_lu     (grid p x 2) the two elimination chains; the bottom one ends
//               with U_M and T'_M
//   k_tw_sweep  (grid p x 2) forward sweeps of the spikes' right-hand sides:
//               W's C^ top-down through L, V's B^ bottom-up through U
//   k_tw_merge  (grid p)     block M: L_M, G_M and X_M of both spikes
//   k_tw_bwd    (grid p x 4) back substitution of W and V, top and bottom halves
//   k_tw_lu_w / k_tw_sweep_w / k_tw_bwd_w   the elimination chains, forward
//               sweeps and back substitution
//               for FP32 16- and 32-row tiles on one warp per chain (TileW), four
//               chains per CTA
//
// Layout, per block J of a partition (factor precision, KB x KB tiles):
//   gL     J <= M: L_J;  J > M: U_J                           (column-major)
//   gG     J <= M: G_J;  J > M: H_J                           (column-major)
//          (T'_M row-major in gG[M] between k_tw_lu and k_tw_merge)
//   gE     J < M: A(J,J+1);  J = M: U_M;  J > M: A(J,J-1)     (column-major)
//   gT     D_J (row-major); A(J,J-1): column-major for J <= M, row-major for
//          J > M; A(J,J+1): row-major for J < M, column-major for J >= M
//          (written by k_band_tiles)
//   gV/gW  row-major forward-sweep scratch, then the column-major spike tiles
// A column-major tile loaded as-is into shared memory is the transposed
// ("At") left operand of Tile::mm_tA.
#include "spike_common.cuh"

#include <type_traits>

namespace {

// global column-major tile -> shared row-major tile (row stride TileLD)
template <class T, int KB, int NT> __device__ __forceinline__ void load_tile_tr(T *s, const T *g)
{
    constexpr int LD = TileLD<T, KB>::value;
    for (int q = threadIdx.x; q < KB * KB; q += NT) {
        const int c = q / KB, r = q - c * KB;
        s[r * LD + c] = g[q];
    }
}

template <class TL, class Reg> __device__ __forceinline__ void rcopy(Reg &d, const Reg &s)
{
#pragma unroll
    for (int i = 0; i < TL::TR; i++)
#pragma unroll
        for (int j = 0; j < TL::TC; j++) d[i][j] = s[i][j];
}

// Shared layout of the two-sided kernels: three tiles, then the mbarriers of
// the tiles that arrive by bulk copies (TwistFits::smem keeps 64 bytes for the
// 16-byte alignment and up to four barriers).
template <class T, class TL> __device__ __forceinline__ uint64_t *tw_bars(char *smraw)
{
    return (uint64_t *)((T *)smem_align(smraw) + 3 * TL::ELEMS);
}

// A timed-out wait (a bulk copy that never landed) ends the kernel in every
// thread at the barrier that follows it: the error word records it, and the
// copies still in flight get their own bounded wait before the CTA leaves.
__device__ __forceinline__ void tw_bail(unsigned *err, TileBar &a, TileBar &b)
{
    if (threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_TIMEOUT);
    a.drain();
    b.drain();
}

// The two elimination chains of each partition (blockIdx.y 0: top, 1: bottom).
// The coupling tiles of the next block arrive by bulk copies while the
// current block's inverse runs, and the next diagonal block by register loads
// issued at the same point, so no step waits on memory.
template <class T, int KB>
__global__ void __launch_bounds__(TwCfg<T, KB>::NT_LU, 4)
    k_tw_lu(const T *__restrict__ gT, const int *__restrict__ blk_off, T *gL, T *gG, T *gE, unsigned *err, int part0)
{
    using TL = typename TwTiles<T, KB>::LU;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x + part0;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * 3 * TS; // per block: D, A(J,J-1), A(J,J+1)

    extern __shared__ char smraw[];
    T *s0 = (T *)smem_align(smraw), *s1 = s0 + TL::ELEMS, *s2 = s1 + TL::ELEMS;
    uint64_t *bars = tw_bars<T, TL>(smraw);
    T *buf = s0; // the inverse's scratch: G_{J-1} / H_{J+1} are consumed before it starts
    TL t(threadIdx.x);
    typename TL::Reg acc, dreg;
    bool ok = true, tmo = false;
    if (threadIdx.x == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init_fence();
    }
    __syncthreads();
    TileBar b1{bars, 0u, false}, b2{bars + 1, 0u, false}; // tiles s1, s2

    if (blockIdx.y == 0) {
        // top chain, J = 0..M-1 (M >= 4)
        T *sG = s0, *sE = s1, *sF = s2;
        b1.issue_dense<T, KB>(sE, gTp + 2 * TS); // A(0,1), row-major (dense: a right operand)
        b2.issue_dense<T, KB>(sF, gTp + 4 * TS); // A(1,0), column-major (dense: a left operand)
        t.gload(acc, gTp);                 // S_0 = D_0
        t.gload(dreg, gTp + 3 * TS);       // D_1
        for (int J = 0; J < M; J++) {
            if (J > 0) {
                tmo |= !b2.wait();
                t.rzero(acc);
                t.template mma_tu<KB, TL::LD>(acc, sF, sG); // L_J; A(J,J-1) is upper triangular
                if (__syncthreads_or(tmo)) return tw_bail(err, b1, b2);
                t.rstore_t(sF, acc);
                t.gstore_t(gL + tb + J * TS, acc);
                tmo |= !b1.wait();
                if (__syncthreads_or(tmo)) return tw_bail(err, b1, b2);
                rcopy<TL>(acc, dreg);
                t.template mms_t_bl<TL::LD, KB>(acc, sF, sE); // S_J = D_J - L_J A(J-1,J); A(J-1,J) lower triangular
                __syncthreads();
                if (J + 1 < M) {
                    b1.issue_dense<T, KB>(sE, gTp + (size_t)J * 3 * TS + 2 * TS);
                    b2.issue_dense<T, KB>(sF, gTp + (size_t)(J + 1) * 3 * TS + TS);
                    t.gload(dreg, gTp + (size_t)(J + 1) * 3 * TS); // D_{J+1}, lands during the inverse
                }
            }
            ok = t.inverse(acc, buf) && ok;
            t.rstore(sG, acc);
            t.gstore_t(gG + tb + J * TS, acc);
            __syncthreads();
        }
    } else {
        // bottom chain, J = N-1..M+1, then U_M and T'_M
        T *sH = s0, *sY = s1, *sX = s2;
        b1.issue_dense<T, KB>(sY, gTp + (size_t)(N - 2) * 3 * TS + 2 * TS); // A(N-2,N-1), column-major
        b2.issue_dense<T, KB>(sX, gTp + (size_t)(N - 1) * 3 * TS + TS);     // A(N-1,N-2), row-major
        t.gload(acc, gTp + (size_t)(N - 1) * 3 * TS);                   // T_{N-1} = D_{N-1}
        t.gload(dreg, gTp + (size_t)(N - 2) * 3 * TS);                  // D_{N-2}
        for (int J = N - 1; J >= M; J--) {
            if (J < N - 1) {
                tmo |= !b1.wait();
                t.rzero(acc);
                t.template mma_tl<KB, TL::LD>(acc, sY, sH); // U_J = A(J,J+1) H_{J+1}; A(J,J+1) lower triangular
                if (__syncthreads_or(tmo)) return tw_bail(err, b1, b2);
                t.rstore_t(sY, acc);
                t.gstore_t((J == M ? gE : gL) + tb + J * TS, acc);
                tmo |= !b2.wait();
                if (__syncthreads_or(tmo)) return tw_bail(err, b1, b2);
                rcopy<TL>(acc, dreg);
                t.template mms_t_bu<TL::LD, KB>(acc, sY, sX); // T_J = D_J - U_J A(J+1,J); A(J+1,J) upper triangular
                if (J == M) {
                    t.gstore(gG + tb + J * TS, acc); // T'_M for k_tw_merge
                    break;
                }
                __syncthreads();
                b1.issue_dense<T, KB>(sY, gTp + (size_t)(J - 1) * 3 * TS + 2 * TS);
                b2.issue_dense<T, KB>(sX, gTp + (size_t)J * 3 * TS + TS);
                t.gload(dreg, gTp + (size_t)(J - 1) * 3 * TS); // D_{J-1}
            }
            ok = t.inverse(acc, buf) && ok;
            t.rstore(sH, acc);
            t.gstore_t(gG + tb + J * TS, acc);
            __syncthreads();
        }
    }
    b1.drain();
    b2.drain();
    if (!ok && threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

// k_tw_lu for FP32 32-row tiles on one warp per chain (TileW): the same two
// elimination chains and the same tiles written, with every tile inverse on
// shuffles.  A CTA holds TW_W_CHAINS independent chains, one per warp, and
// nothing synchronizes across warps.  Per warp, three dense shared tiles: s0
// holds G_{J-1} / H_{J+1} and then the product L_J / U_J (as a left
// operand); s1 and s2 take the bulk copies.  The diagonal block D_J arrives by
// bulk copy into the buffer of the coupling tile the first product has just
// consumed, so no tile waits in registers.
constexpr int TW_W_CHAINS = 4; // chains (warps) per CTA of k_tw_lu_w

// one shared tile's barrier as the lanes of one warp track it (the warp's
// lane 0 issues the copy); the warp form of TileBar
struct WarpBar {
    uint64_t *bar;
    unsigned phase;
    bool inflight;
    template <class T, int KB> __device__ __forceinline__ void issue(T *s, const T *g)
    {
        __syncwarp();
        bulk_tile_dense<T, KB>(s, g, bar);
        inflight = true;
    }
    __device__ __forceinline__ bool wait()
    {
        const bool ok = mbar_wait(bar, phase);
        phase ^= 1u;
        inflight = false;
        return ok;
    }
    __device__ __forceinline__ void drain()
    {
        if (inflight) wait();
    }
};

__device__ __forceinline__ void tw_bail_w(unsigned *err, WarpBar &a, WarpBar &b)
{
    if ((threadIdx.x & 31) == 0) atomicOr(err, SPK_DEV_ERR_TIMEOUT);
    a.drain();
    b.drain();
}

template <class T, int KB>
__global__ void __launch_bounds__(32 * TW_W_CHAINS)
    k_tw_lu_w(const T *__restrict__ gT, const int *__restrict__ blk_off, T *gL, T *gG, T *gE, unsigned *err,
              int part0, int np)
{
    using TL = TileW<T, KB>;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr size_t TS = (size_t)KB * KB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chain = blockIdx.x * TW_W_CHAINS + warp;
    if (chain >= 2 * np) return; // the whole warp
    const int part = (chain >> 1) + part0;
    const bool top = (chain & 1) == 0;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * 3 * TS; // per block: D, A(J,J-1), A(J,J+1)

    extern __shared__ char smraw[];
    T *base = (T *)smem_align(smraw);
    T *s0 = base + (size_t)warp * 3 * TL::ELEMS, *s1 = s0 + TL::ELEMS, *s2 = s1 + TL::ELEMS;
    uint64_t *bars = (uint64_t *)(base + (size_t)TW_W_CHAINS * 3 * TL::ELEMS) + 2 * warp;
    TL t(lane);
    typename TL::Reg acc;
    bool ok = true, tmo = false;
    if (lane == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init_fence();
    }
    __syncwarp();
    WarpBar b1{bars, 0u, false}, b2{bars + 1, 0u, false}; // tiles s1, s2

    if (top) {
        // top chain, J = 0..M-1 (M >= 4)
        T *sG = s0, *sE = s1, *sX = s2;
        b1.issue<T, KB>(sE, gTp + 2 * TS); // A(0,1), row-major: the right operand of S_1
        b2.issue<T, KB>(sX, gTp + 4 * TS); // A(1,0), column-major: the left operand of L_1
        t.gload(acc, gTp);                 // S_0 = D_0
        for (int J = 0; J < M; J++) {
            if (J > 0) {
                tmo |= !b2.wait();
                if (__any_sync(FULL, tmo)) return tw_bail_w(err, b1, b2);
                t.rzero(acc);
                t.template mm_tA<false>(acc, sX, sG); // L_J = A(J,J-1) G_{J-1}
                b2.issue<T, KB>(sX, gTp + (size_t)J * 3 * TS); // D_J, lands during the next product
                t.rstore_t(sG, acc);
                t.gstore_t(gL + tb + J * TS, acc);
                tmo |= !b1.wait();
                if (__any_sync(FULL, tmo)) return tw_bail_w(err, b1, b2);
                __syncwarp(); // L_J's shared image is complete
                t.rzero(acc);
                t.template mm_tA<true>(acc, sG, sE); // - L_J A(J-1,J)
                tmo |= !b2.wait();
                if (__any_sync(FULL, tmo)) return tw_bail_w(err, b1, b2);
                t.radd(acc, sX); // S_J = D_J - L_J A(J-1,J)
                if (J + 1 < M) {
                    b1.issue<T, KB>(sE, gTp + (size_t)J * 3 * TS + 2 * TS);
                    b2.issue<T, KB>(sX, gTp + (size_t)(J + 1) * 3 * TS + TS);
                }
            }
            ok = t.inverse(acc) && ok;
            __syncwarp();
            t.rstore(sG, acc);
            t.gstore_t(gG + tb + J * TS, acc);
            __syncwarp();
        }
    } else {
        // bottom chain, J = N-1..M+1, then U_M and T'_M
        T *sH = s0, *sY = s1, *sX = s2;
        b1.issue<T, KB>(sY, gTp + (size_t)(N - 2) * 3 * TS + 2 * TS); // A(N-2,N-1), column-major
        b2.issue<T, KB>(sX, gTp + (size_t)(N - 1) * 3 * TS + TS);     // A(N-1,N-2), row-major
        t.gload(acc, gTp + (size_t)(N - 1) * 3 * TS);                  // T_{N-1} = D_{N-1}
        for (int J = N - 1; J >= M; J--) {
            if (J < N - 1) {
                tmo |= !b1.wait();
                if (__any_sync(FULL, tmo)) return tw_bail_w(err, b1, b2);
                t.rzero(acc);
                t.template mm_tA<false>(acc, sY, sH); // U_J = A(J,J+1) H_{J+1}
                b1.issue<T, KB>(sY, gTp + (size_t)J * 3 * TS); // D_J, lands during the next product
                t.rstore_t(sH, acc);
                t.gstore_t((J == M ? gE : gL) + tb + J * TS, acc);
                tmo |= !b2.wait();
                if (__any_sync(FULL, tmo)) return tw_bail_w(err, b1, b2);
                __syncwarp(); // U_J's shared image is complete
                t.rzero(acc);
                t.template mm_tA<true>(acc, sH, sX); // - U_J A(J+1,J)
                tmo |= !b1.wait();
                if (__any_sync(FULL, tmo)) return tw_bail_w(err, b1, b2);
                t.radd(acc, sY); // T_J = D_J - U_J A(J+1,J)
                if (J == M) {
                    t.gstore(gG + tb + J * TS, acc); // T'_M for k_tw_merge
                    break;
                }
                b1.issue<T, KB>(sY, gTp + (size_t)(J - 1) * 3 * TS + 2 * TS);
                b2.issue<T, KB>(sX, gTp + (size_t)J * 3 * TS + TS);
            }
            ok = t.inverse(acc) && ok;
            __syncwarp();
            t.rstore(sH, acc);
            t.gstore_t(gG + tb + J * TS, acc);
            __syncwarp();
        }
    }
    b1.drain();
    b2.drain();
    if (!ok && lane == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}
// k_tw_bwd on one warp per chain (TileW): the back substitution of W and V
// from X_M outwards, chain c of a CTA's TW_W_CHAINS taking (partition c / 4,
// spike half c % 4) in k_tw_bwd's numbering (0 W top, 1 W bottom, 2 V top,
// 3 V bottom).  Per warp, the tiles G_J / H_J and the coupling tile arrive by
// bulk copies; X stays in a dense shared tile as the right operand.
template <class T, int KB>
__global__ void __launch_bounds__(32 * TW_W_CHAINS)
    k_tw_bwd_w(const int *__restrict__ blk_off, int p, const T *__restrict__ gG, const T *__restrict__ gE, T *gV,
               T *gW, int part0, int np, unsigned *err)
{
    using TL = TileW<T, KB>;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr size_t TS = (size_t)KB * KB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chain = blockIdx.x * TW_W_CHAINS + warp;
    if (chain >= 4 * np) return; // the whole warp
    const int part = (chain >> 2) + part0, which = chain & 3;
    const bool isV = which >= 2, top = (which & 1) == 0;
    if (isV ? part == p - 1 : part == 0) return; // no such spike
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    T *gX = isV ? gV : gW;
    const bool hasZ = isV ? !top : top;
    const int cnt = top ? M : N - 1 - M;

    extern __shared__ char smraw[];
    T *base = (T *)smem_align(smraw);
    T *sG = base + (size_t)warp * 3 * TL::ELEMS, *sE = sG + TL::ELEMS, *sX = sE + TL::ELEMS;
    uint64_t *bars = (uint64_t *)(base + (size_t)TW_W_CHAINS * 3 * TL::ELEMS) + 2 * warp;
    TL t(lane);
    typename TL::Reg acc, zreg;
    if (lane == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init_fence();
    }
    __syncwarp();
    WarpBar bG{bars, 0u, false}, bE{bars + 1, 0u, false};
    bool tmo = false;

    const int J1 = top ? M - 1 : M + 1;
    bG.issue<T, KB>(sG, gG + tb + (size_t)J1 * TS); // left operands: dense
    bE.issue<T, KB>(sE, gE + tb + (size_t)J1 * TS);
    if (hasZ) t.gload(zreg, gX + tb + (size_t)J1 * TS); // Z_J of the first step (row-major)
    {
        // X_M (column-major in global) -> the lane's sub-tile -> a row-major dense tile
        const T *gm = gX + tb + (size_t)M * TS;
#pragma unroll
        for (int j = 0; j < TL::TC; j++) {
            T c[TL::TR];
            vld<T, TL::TR>(c, gm + (size_t)t.col(j) * KB + t.row(0));
#pragma unroll
            for (int i = 0; i < TL::TR; i++) acc[i][j] = c[i];
        }
        t.rstore(sX, acc);
    }
    __syncwarp();
    for (int i = 0; i < cnt; i++) {
        const int J = top ? M - 1 - i : M + 1 + i;
        const int Jn = top ? J - 1 : J + 1;
        const bool more = i + 1 < cnt;
        if (hasZ) {
#pragma unroll
            for (int r = 0; r < TL::TR; r++)
#pragma unroll
                for (int c = 0; c < TL::TC; c++) acc[r][c] = zreg[r][c];
        } else {
            t.rzero(acc);
        }
        tmo |= !bE.wait();
        if (__any_sync(FULL, tmo)) return tw_bail_w(err, bG, bE);
        t.template mm_tA<true>(acc, sE, sX); // Z_J - A(J,J+-1) X_{J+-1}
        if (more) bE.issue<T, KB>(sE, gE + tb + (size_t)Jn * TS); // (syncs the warp: sX reads done)
        else
            __syncwarp();
        t.rstore(sX, acc);
        if (hasZ && more) t.gload(zreg, gX + tb + (size_t)Jn * TS); // Z of the next step, lands meanwhile
        tmo |= !bG.wait();
        if (__any_sync(FULL, tmo)) return tw_bail_w(err, bG, bE);
        __syncwarp(); // the updated right-hand side is in sX
        t.rzero(acc);
        t.template mm_tA<false>(acc, sG, sX); // X_J = G_J (...)
        if (more) bG.issue<T, KB>(sG, gG + tb + (size_t)Jn * TS);
        else
            __syncwarp();
        t.rstore(sX, acc);
        t.gstore_t(gX + tb + (size_t)J * TS, acc);
        __syncwarp();
    }
    bG.drain();
    bE.drain();
}

// shared bytes of k_tw_lu_w: three dense tiles and two mbarriers per chain,
// alignment
template <class T, int KB> constexpr size_t tw_lu_w_smem()
{
    return (size_t)TW_W_CHAINS * 3 * sizeof(T) * KB * KB + 16 * TW_W_CHAINS + 16;
}
// FP32 16- and 32-row tiles take the one-warp elimination chains
template <class T, int KB> constexpr bool tw_lu_w_ok() { return sizeof(T) == 4 && (KB == 16 || KB == 32); }

// V's right-hand side [0; B^] restricted to block J: B^ fills the last KB
// real rows of the partition, i.e. rows o..KB-1 of block J0 and rows 0..o-1
// of block J0+1 (when o > 0).
template <class T, int KB, class TL>
__device__ __forceinline__ void bhat_block(const TL &t, typename TL::Reg &a, const T *bh, int J, int J0, int o)
{
#pragma unroll
    for (int i = 0; i < TL::TR; i++)
#pragma unroll
        for (int j = 0; j < TL::TC; j++) {
            const int r = t.row(i), c = t.col(j);
            T v = sc_zero<T>();
            if (t.act) {
                if (J == J0 && r >= o)
                    v = bh[(r - o) * KB + c];
                else if (o > 0 && J == J0 + 1 && r < o)
                    v = bh[(KB - o + r) * KB + c];
            }
            a[i][j] = v;
        }
}

// k_tw_sweep on one warp per chain (TileW): the spikes' forward sweeps, W's
// C^ top-down through L and V's B^ bottom-up through U, chain c of a CTA
// taking (partition c / 2, top or bottom).  The factor tiles of consecutive
// blocks alternate between two dense shared tiles filled by bulk copies one
// block ahead; z stays in a third as the right operand.
template <class T, int KB>
__global__ void __launch_bounds__(32 * TW_W_CHAINS)
    k_tw_sweep_w(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                 const T *__restrict__ gL, const T *__restrict__ gE, const T *__restrict__ gBhat, T *gV, T *gW,
                 int part0, int np, unsigned *err)
{
    using TL = TileW<T, KB>;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr size_t TS = (size_t)KB * KB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chain = blockIdx.x * TW_W_CHAINS + warp;
    if (chain >= 2 * np) return; // the whole warp
    const int part = (chain >> 1) + part0;
    const bool top = (chain & 1) == 0;
    if (top ? part == 0 : part == p - 1) return; // no such spike
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;

    extern __shared__ char smraw[];
    T *base = (T *)smem_align(smraw);
    T *sZ = base + (size_t)warp * 3 * TL::ELEMS, *sA = sZ + TL::ELEMS, *sB = sA + TL::ELEMS;
    uint64_t *bars = (uint64_t *)(base + (size_t)TW_W_CHAINS * 3 * TL::ELEMS) + 3 * warp;
    TL t(lane);
    typename TL::Reg acc;
    if (lane == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init(bars + 2, 1);
        mbar_init_fence();
    }
    __syncwarp();
    WarpBar bA{bars, 0u, false}, bB{bars + 1, 0u, false}, bZ{bars + 2, 0u, false};
    auto ring = [&](int J) { return (J & 1) ? sB : sA; };
    auto rbar = [&](int J) -> WarpBar & { return (J & 1) ? bB : bA; };
    auto bail = [&] {
        if (lane == 0) atomicOr(err, SPK_DEV_ERR_TIMEOUT);
        bA.drain();
        bB.drain();
        bZ.drain();
    };
    bool tmo = false;

    if (top) {
        // W: z_0 = C^ (gW tile 0, from the band pass), z_J = -L_J z_{J-1}, J = 1..M-1
        bZ.issue<T, KB>(sZ, gW + tb);
        rbar(1).template issue<T, KB>(ring(1), gL + tb + TS);
        tmo |= !bZ.wait();
        if (__any_sync(FULL, tmo)) return bail();
        for (int J = 1; J < M; J++) {
            if (J + 1 < M) rbar(J + 1).template issue<T, KB>(ring(J + 1), gL + tb + (size_t)(J + 1) * TS);
            tmo |= !rbar(J).wait();
            if (__any_sync(FULL, tmo)) return bail();
            t.rzero(acc);
            t.template mm_tA<true>(acc, ring(J), sZ);
            __syncwarp(); // every lane has read z_{J-1}
            t.rstore(sZ, acc);
            t.gstore(gW + tb + (size_t)J * TS, acc);
            __syncwarp();
        }
    } else {
        // V: w_J = r_J - U_J w_{J+1}, J = N-1..M (U_M lives in gE)
        const int m = part_start[part + 1] - part_start[part];
        const int J0 = (m - KB) / KB, o = (m - KB) - J0 * KB; // m >= 8 KB: o >= 0, J0 > M
        const T *bh = gBhat + (size_t)part * TS;
        auto utile = [&](int J) { return (J == M ? gE : gL) + tb + (size_t)J * TS; };
        rbar(N - 2).template issue<T, KB>(ring(N - 2), utile(N - 2));
        bhat_block<T, KB>(t, acc, bh, N - 1, J0, o);
        t.rstore(sZ, acc);
        t.gstore(gV + tb + (size_t)(N - 1) * TS, acc);
        __syncwarp();
        for (int J = N - 2; J >= M; J--) {
            if (J - 1 >= M) rbar(J - 1).template issue<T, KB>(ring(J - 1), utile(J - 1));
            bhat_block<T, KB>(t, acc, bh, J, J0, o);
            tmo |= !rbar(J).wait();
            if (__any_sync(FULL, tmo)) return bail();
            t.template mm_tA<true>(acc, ring(J), sZ);
            __syncwarp(); // every lane has read w_{J+1}
            t.rstore(sZ, acc);
            t.gstore(gV + tb + (size_t)J * TS, acc);
            __syncwarp();
        }
    }
    bA.drain();
    bB.drain();
    bZ.drain();
}
// shared bytes of k_tw_sweep_w: three dense tiles and three mbarriers per
// chain, alignment
template <class T, int KB> constexpr size_t tw_sweep_w_smem()
{
    return (size_t)TW_W_CHAINS * 3 * sizeof(T) * KB * KB + 24 * TW_W_CHAINS + 16;
}

// The spikes' forward sweeps.  The factor tiles of consecutive blocks
// alternate between two shared buffers (sA: even J, sB: odd J), each filled by
// bulk copies one block ahead; the parity of a buffer's phase follows from J.
template <class T, int KB>
__global__ void __launch_bounds__(TwCfg<T, KB>::NT_PROD, 4)
    k_tw_sweep(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p, const T *__restrict__ gL,
               const T *__restrict__ gE, const T *__restrict__ gBhat, T *gV, T *gW, int part0, unsigned *err)
{
    using TL = typename TwTiles<T, KB>::PROD;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x + part0;
    const bool top = blockIdx.y == 0;
    if (top ? part == 0 : part == p - 1) return; // the whole CTA: no such spike
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;

    extern __shared__ char smraw[];
    T *sZ = (T *)smem_align(smraw), *sA = sZ + TL::ELEMS, *sB = sA + TL::ELEMS;
    uint64_t *bars = tw_bars<T, TL>(smraw); // [0] sA, [1] sB, [2] sZ
    TL t(threadIdx.x);
    typename TL::Reg acc;
    if (threadIdx.x == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init(bars + 2, 1);
        mbar_init_fence();
    }
    __syncthreads();
    bool tmo = false;
    // ring buffer of block J and the parity of its wait for block J
    auto ring = [&](int J) { return (J & 1) ? sB : sA; };
    auto issue = [&](int J, const T *g) {
        if (threadIdx.x < 32) bulk_tile_dense<T, KB>(ring(J), g, bars + (J & 1));
    };
    auto bail = [&](int Jn, unsigned ph) { // a copy for block Jn may be in flight
        if (threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_TIMEOUT);
        if (Jn >= 0) mbar_wait(bars + (Jn & 1), ph);
    };

    if (top) {
        // W: z_0 = C^ (gW tile 0, from k_band_tiles), z_J = -L_J z_{J-1}, J = 1..M-1
        if (threadIdx.x < 32) bulk_tile<T, KB>(sZ, gW + tb, bars + 2);
        issue(1, gL + tb + TS);
        tmo |= !mbar_wait(bars + 2, 0);
        for (int J = 1; J < M; J++) {
            const bool more = J + 1 < M;
            if (more) issue(J + 1, gL + tb + (size_t)(J + 1) * TS);
            tmo |= !mbar_wait(bars + (J & 1), ((J - 1) >> 1) & 1);
            t.rzero(acc);
            t.template mms_t<KB, TL::LD>(acc, ring(J), sZ);
            if (__syncthreads_or(tmo)) return bail(more ? J + 1 : -1, (J >> 1) & 1);
            t.rstore(sZ, acc);
            t.gstore(gW + tb + J * TS, acc);
            __syncthreads();
        }
    } else {
        // V: w_J = r_J - U_J w_{J+1}, J = N-1..M (U_M lives in gE)
        const int m = part_start[part + 1] - part_start[part];
        const int J0 = (m - KB) / KB, o = (m - KB) - J0 * KB; // m >= 8 KB: o >= 0, J0 > M
        const T *bh = gBhat + (size_t)part * TS;
        auto utile = [&](int J) { return (J == M ? gE : gL) + tb + (size_t)J * TS; };
        auto phase = [&](int J) { return (unsigned)(((N - 2 - J) >> 1) & 1); };
        issue(N - 2, utile(N - 2));
        bhat_block<T, KB>(t, acc, bh, N - 1, J0, o);
        t.rstore(sZ, acc);
        t.gstore(gV + tb + (size_t)(N - 1) * TS, acc);
        __syncthreads();
        for (int J = N - 2; J >= M; J--) {
            const bool more = J - 1 >= M;
            if (more) issue(J - 1, utile(J - 1));
            bhat_block<T, KB>(t, acc, bh, J, J0, o);
            tmo |= !mbar_wait(bars + (J & 1), phase(J));
            t.template mms_t<KB, TL::LD>(acc, ring(J), sZ);
            if (__syncthreads_or(tmo)) return bail(more ? J - 1 : -1, phase(J - 1));
            t.rstore(sZ, acc);
            t.gstore(gV + tb + J * TS, acc);
            __syncthreads();
        }
    }
}

template <class T, int KB>
__global__ void __launch_bounds__(TwCfg<T, KB>::NT_LU, 4)
    k_tw_merge(const T *__restrict__ gT, const int *__restrict__ blk_off, int p, T *gL, T *gG, T *gV, T *gW,
               unsigned *err, int part0)
{
    constexpr int NT = TwCfg<T, KB>::NT_LU;
    using TL = typename TwTiles<T, KB>::LU;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x + part0;
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * 3 * TS;

    extern __shared__ char smraw[];
    T *sA = (T *)smem_align(smraw), *sB = sA + TL::ELEMS, *sC = sB + TL::ELEMS;
    T *buf = sA; // the inverse's scratch: G_{M-1} is consumed before it starts
    TL t(threadIdx.x);
    typename TL::Reg acc;

    cp_async_tile<T, KB, NT>(sC, gTp + (size_t)M * 3 * TS + TS);           // A(M,M-1), column-major
    cp_async_tile<T, KB, NT>(sB, gTp + (size_t)(M - 1) * 3 * TS + 2 * TS); // A(M-1,M), row-major
    cp_async_commit();
    load_tile_tr<T, KB, NT>(sA, gG + tb + (size_t)(M - 1) * TS);            // G_{M-1}, row-major
    cp_async_wait_all();
    __syncthreads();
    t.rzero(acc);
    t.mma_tu(acc, sC, sA); // L_M
    __syncthreads();
    t.rstore_t(sC, acc);
    t.gstore_t(gL + tb + M * TS, acc);
    __syncthreads();
    t.gload(acc, gG + tb + M * TS); // T'_M
    t.mms_t_bl(acc, sC, sB);        // S_M = T'_M - L_M A(M-1,M) (lower triangular)
    const bool ok = t.inverse(acc, buf);
    t.rstore_t(sA, acc); // G_M as a left operand
    t.gstore_t(gG + tb + M * TS, acc);
    __syncthreads();
    if (part > 0) {
        // W: z_M = -L_M z_{M-1} (its bottom half is zero), X_M = G_M z_M
        cp_async_tile<T, KB, NT>(sB, gW + tb + (size_t)(M - 1) * TS);
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        t.rzero(acc);
        t.mms_t(acc, sC, sB);
        __syncthreads();
        t.rstore(sB, acc);
        __syncthreads();
        t.rzero(acc);
        t.mma_t(acc, sA, sB);
        t.gstore_t(gW + tb + M * TS, acc);
        __syncthreads();
    }
    if (part < p - 1) {
        // V: z_M = w_M (its top half is zero), X_M = G_M w_M
        cp_async_tile<T, KB, NT>(sB, gV + tb + (size_t)M * TS);
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        t.rzero(acc);
        t.mma_t(acc, sA, sB);
        t.gstore_t(gV + tb + M * TS, acc);
    }
    if (!ok && threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

// Back substitution from X_M outwards; blockIdx.y: 0 W top, 1 W bottom,
// 2 V top, 3 V bottom.
//   top     X_J = G_J (Z_J - A(J,J+1) X_{J+1}),  J = M-1..0
//   bottom  X_J = H_J (Z_J - A(J,J-1) X_{J-1}),  J = M+1..N-1
// Z_J is the forward sweep where the spike has one (W's top half, V's bottom
// half), else zero.
template <class T, int KB>
__global__ void __launch_bounds__(TwCfg<T, KB>::NT_PROD, 4)
    k_tw_bwd(const int *__restrict__ blk_off, int p, const T *__restrict__ gG, const T *__restrict__ gE, T *gV,
             T *gW, int part0, unsigned *err)
{
    constexpr int NT = TwCfg<T, KB>::NT_PROD;
    using TL = typename TwTiles<T, KB>::PROD;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x + part0, which = blockIdx.y;
    const bool isV = which >= 2, top = (which & 1) == 0;
    if (isV ? part == p - 1 : part == 0) return; // the whole CTA: no such spike
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    T *gX = isV ? gV : gW;
    const bool hasZ = isV ? !top : top;
    const int cnt = top ? M : N - 1 - M;

    extern __shared__ char smraw[];
    T *sG = (T *)smem_align(smraw), *sE = sG + TL::ELEMS, *sX = sE + TL::ELEMS;
    uint64_t *bars = tw_bars<T, TL>(smraw);
    TL t(threadIdx.x);
    typename TL::Reg acc, zreg;
    if (threadIdx.x == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init_fence();
    }
    __syncthreads();
    TileBar bG{bars, 0u, false}, bE{bars + 1, 0u, false};
    bool tmo = false;

    const int J1 = top ? M - 1 : M + 1;
    bG.issue_dense<T, KB>(sG, gG + tb + (size_t)J1 * TS); // left operands: dense
    bE.issue_dense<T, KB>(sE, gE + tb + (size_t)J1 * TS);
    if (hasZ) t.gload(zreg, gX + tb + (size_t)J1 * TS); // Z_J of the first step
    load_tile_tr<T, KB, NT>(sX, gX + tb + (size_t)M * TS); // X_M, row-major
    __syncthreads();
    for (int i = 0; i < cnt; i++) {
        const int J = top ? M - 1 - i : M + 1 + i;
        const int Jn = top ? J - 1 : J + 1;
        const bool more = i + 1 < cnt;
        if (hasZ)
            rcopy<TL>(acc, zreg);
        else
            t.rzero(acc);
        tmo |= !bE.wait();
        if (top)
            t.template mms_tl<KB, TL::LD>(acc, sE, sX); // A(J,J+1) lower triangular
        else
            t.template mms_tu<KB, TL::LD>(acc, sE, sX); // A(J,J-1) upper triangular
        if (__syncthreads_or(tmo)) return tw_bail(err, bG, bE);
        if (more) bE.issue_dense<T, KB>(sE, gE + tb + (size_t)Jn * TS);
        t.rstore(sX, acc);
        if (hasZ && more) t.gload(zreg, gX + tb + (size_t)Jn * TS); // Z of the next step, lands meanwhile
        tmo |= !bG.wait();
        if (__syncthreads_or(tmo)) return tw_bail(err, bG, bE);
        t.rzero(acc);
        t.template mma_t<KB, TL::LD>(acc, sG, sX);
        __syncthreads();
        if (more) bG.issue_dense<T, KB>(sG, gG + tb + (size_t)Jn * TS);
        t.rstore(sX, acc);
        t.gstore_t(gX + tb + (size_t)J * TS, acc);
        __syncthreads();
    }
    bG.drain();
    bE.drain();
}

// ------------------------------------------------------------ small bands
// KB <= 4: the same two-sided recurrences on KB lanes per chain (lane r owns
// row r of every tile; the other rows arrive by shuffles), with each chain's
// next blocks streaming into its own shared-memory ring, as k_quad_fwd /
// k_quad_bwd.  Here the W forward sweep rides along the top elimination
// chain and V's forward sweep along the bottom one.
template <class T, int KB> struct QTw {
    static constexpr int TS = KB * KB;
    static constexpr int EL = KB * KB;                               // lanes per chain: one tile element each
    static constexpr int DEPTH = 4;
    static constexpr int STAGE = 3 * TS;                             // three tiles per block
    static constexpr int SLOT = DEPTH * STAGE * (int)sizeof(T) + 16; // per chain
    static constexpr int CPC = 256 / EL;                             // chains per CTA, at most
    static constexpr int NT = CPC * EL;
    static constexpr size_t SMEM = (size_t)CPC * SLOT;
};

// The first half of the grid runs the top chains, the second half the
// bottom chains, so a warp never holds both: their loops differ, and a warp
// with both would step through one and then the other.  A chain takes KB*KB
// lanes, lane (r, c) holding element (r, c) of each tile (el_mul, el_inv).
template <class T, int KB>
__global__ void __launch_bounds__(QTw<T, KB>::NT)
    k_qtw_lu(const T *__restrict__ gT, const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
             const T *__restrict__ gBhat, T *gL, T *gG, T *gE, T *gV, T *gW, unsigned *err)
{
    using C = QTw<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH, EL = C::EL;
    constexpr int CH = C::STAGE * (int)sizeof(T) / 16;
    extern __shared__ __align__(16) char smc[];
    const int half_grid = (int)gridDim.x / 2; // CTAs per direction
    const bool bottom = (int)blockIdx.x >= half_grid;
    const int part = ((int)blockIdx.x - (bottom ? half_grid : 0)) * ((int)blockDim.x / EL) + (int)threadIdx.x / EL;
    const int e = threadIdx.x % EL, r = e / KB, c = e % KB;
    if (part >= p) return; // whole segments leave together; no CTA barriers below
    const unsigned m = seg_mask<EL>();
    T *slot = (T *)(smc + (threadIdx.x / EL) * C::SLOT);
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * C::STAGE;
    const int cnt = bottom ? N - M : M;
    auto issue = [&](int i) {
        if (i < cnt) {
            const int J = bottom ? N - 1 - i : i;
            for (int q = e; q < CH; q += EL)
                cp_async16((char *)(slot + (i % D) * C::STAGE) + 16 * q,
                           (const char *)(gTp + (size_t)J * C::STAGE) + 16 * q);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int i = 0; i < D - 1; i++) issue(i);
    bool ok = true;
    const int rm = r * KB + c, cm = c * KB + r; // element (r, c) of a row-major / column-major tile
    if (!bottom) {
        // L_J = A(J,J-1) G_{J-1}, S_J = D_J - L_J A(J-1,J), G_J = S_J^{-1}; z_J = -L_J z_{J-1}
        const bool doW = part > 0;
        T g = sc_zero<T>(), ep = sc_zero<T>();
        T zp = doW ? gW[tb + rm] : sc_zero<T>(); // z_0 = C^
        for (int J = 0; J < cnt; J++) {
            issue(J + D - 1);
            cp_async_wait_n<D - 1>();
            __syncwarp(m);
            const T *sc = slot + (J % D) * C::STAGE;
            T sv = sc[rm]; // D_J
            if (J > 0) {
                const T l = el_mul<T, KB>(m, sc[TS + cm], g, r, c); // A(J,J-1) is column-major
                gL[tb + (size_t)J * TS + cm] = l;
                sv = el_msub<T, KB>(m, sv, l, ep, r, c);
                if (doW) {
                    zp = el_msub<T, KB>(m, sc_zero<T>(), l, zp, r, c);
                    gW[tb + (size_t)J * TS + rm] = zp;
                }
            }
            ep = sc[2 * TS + rm]; // A(J,J+1), row-major
            __syncwarp(m);        // the ring entry may be refilled from here on
            ok = el_inv<T, KB>(m, sv, r, c) && ok;
            gG[tb + (size_t)J * TS + cm] = sv;
            g = sv;
        }
    } else {
        // U_J = A(J,J+1) H_{J+1}, T_J = D_J - U_J A(J+1,J), H_J = T_J^{-1}; w_J = r_J - U_J w_{J+1}
        // with V's right-hand side r = [0; B^] in blocks J0 (rows o..KB-1) and
        // J0+1 (rows 0..o-1); every partition has >= 8 blocks, so J0 > M
        const bool doV = part < p - 1;
        const int mrows = part_start[part + 1] - part_start[part];
        const int J0 = (mrows - KB) / KB, o = mrows - KB - J0 * KB;
        const T *B = gBhat + (size_t)part * TS;
        T h = sc_zero<T>(), xn = sc_zero<T>(), wp = sc_zero<T>();
        for (int i = 0; i < cnt; i++) {
            const int J = N - 1 - i;
            issue(i + D - 1);
            cp_async_wait_n<D - 1>();
            __syncwarp(m);
            const T *sc = slot + (i % D) * C::STAGE;
            T sv = sc[rm]; // D_J
            T rv = (J == J0 && r >= o) ? B[(r - o) * KB + c]
                                       : (o > 0 && J == J0 + 1 && r < o) ? B[(KB - o + r) * KB + c] : sc_zero<T>();
            if (i > 0) {
                const T u = el_mul<T, KB>(m, sc[2 * TS + cm], h, r, c); // A(J,J+1) is column-major here
                ((J == M ? gE : gL) + tb + (size_t)J * TS)[cm] = u;
                sv = el_msub<T, KB>(m, sv, u, xn, r, c);
                if (doV) rv = el_msub<T, KB>(m, rv, u, wp, r, c);
            }
            if (doV) {
                gV[tb + (size_t)J * TS + rm] = rv;
                wp = rv;
            }
            if (J == M) { // T'_M for the middle block, row-major
                gG[tb + (size_t)J * TS + rm] = sv;
                break;
            }
            xn = sc[TS + rm]; // A(J,J-1), row-major
            __syncwarp(m);
            ok = el_inv<T, KB>(m, sv, r, c) && ok;
            gG[tb + (size_t)J * TS + cm] = sv;
            h = sv;
        }
    }
    cp_async_wait_all();
    if (!ok && e == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

// the middle block of every partition (KB lanes each): L_M, G_M, and X_M of W and V
template <class T, int KB>
__global__ void k_qtw_merge(const T *__restrict__ gT, const int *__restrict__ blk_off, int p, T *gL, T *gG, T *gV,
                            T *gW, unsigned *err)
{
    constexpr int TS = KB * KB;
    const int part = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int r = threadIdx.x % KB;
    if (part >= p) return; // whole segments
    const unsigned m = seg_mask<KB>();
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * 3 * TS;
    T f[KB], g[KB], l[KB], sr[KB], ep[KB], zp[KB], w[KB];
#pragma unroll
    for (int c = 0; c < KB; c++) {
        f[c] = gTp[(size_t)M * 3 * TS + TS + c * KB + r];           // row r of A(M,M-1) (column-major)
        g[c] = gG[tb + (size_t)(M - 1) * TS + c * KB + r];           // row r of G_{M-1}
        sr[c] = gG[tb + (size_t)M * TS + r * KB + c];                // row r of T'_M (row-major)
        ep[c] = gTp[(size_t)(M - 1) * 3 * TS + 2 * TS + r * KB + c]; // row r of A(M-1,M) (row-major)
        zp[c] = part > 0 ? gW[tb + (size_t)(M - 1) * TS + r * KB + c] : sc_zero<T>();
        w[c] = part < p - 1 ? gV[tb + (size_t)M * TS + r * KB + c] : sc_zero<T>();
    }
    row_mul<T, KB>(m, l, f, g); // L_M
    row_msub<T, KB>(m, sr, l, ep);
    const bool ok = row_inv<T, KB>(m, sr, r); // G_M
    __syncwarp(m); // every lane has read its rows of T'_M and w_M before they are overwritten
#pragma unroll
    for (int c = 0; c < KB; c++) {
        gL[tb + (size_t)M * TS + c * KB + r] = l[c];
        gG[tb + (size_t)M * TS + c * KB + r] = sr[c];
    }
    if (part > 0) { // W: z_M = -L_M z_{M-1}, X_M = G_M z_M
        T z[KB], x[KB];
#pragma unroll
        for (int c = 0; c < KB; c++) z[c] = sc_zero<T>();
        row_msub<T, KB>(m, z, l, zp);
        row_mul<T, KB>(m, x, sr, z);
#pragma unroll
        for (int c = 0; c < KB; c++) gW[tb + (size_t)M * TS + c * KB + r] = x[c];
    }
    if (part < p - 1) { // V: X_M = G_M w_M
        T x[KB];
        row_mul<T, KB>(m, x, sr, w);
#pragma unroll
        for (int c = 0; c < KB; c++) gV[tb + (size_t)M * TS + c * KB + r] = x[c];
    }
    if (!ok && r == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

// back substitution from X_M outwards; chain 4*part + {0: W top, 1: W bottom,
// 2: V top, 3: V bottom}; the ring holds G or H, the coupling tile and Z
template <class T, int KB>
__global__ void __launch_bounds__(QTw<T, KB>::NT)
    k_qtw_bwd(const int *__restrict__ blk_off, int p, const T *__restrict__ gG, const T *__restrict__ gE, T *gV,
              T *gW)
{
    using C = QTw<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH, EL = C::EL;
    constexpr int CT = TS * (int)sizeof(T) / 16;
    extern __shared__ __align__(16) char smc[];
    const int ch = (blockIdx.x * blockDim.x + threadIdx.x) / EL;
    const int e = threadIdx.x % EL, r = e / KB, c = e % KB;
    const int part = ch >> 2, which = ch & 3;
    const bool isV = which >= 2, top = (which & 1) == 0;
    if (part >= p || (isV ? part == p - 1 : part == 0)) return; // whole segments
    const unsigned m = seg_mask<EL>();
    T *slot = (T *)(smc + (threadIdx.x / EL) * C::SLOT);
    const int N = blk_off[part + 1] - blk_off[part], M = N / 2;
    const size_t tb = (size_t)blk_off[part] * TS;
    T *gX = isV ? gV : gW;
    const bool hasZ = isV ? !top : top;
    const int cnt = top ? M : N - 1 - M;
    const int rm = r * KB + c, cm = c * KB + r;
    auto blk = [&](int i) { return top ? M - 1 - i : M + 1 + i; };
    auto issue = [&](int i) {
        if (i < cnt) {
            const int J = blk(i);
            char *st = (char *)(slot + (i % D) * C::STAGE);
            for (int q = e; q < CT; q += EL) {
                cp_async16(st + 16 * q, (const char *)(gG + tb + (size_t)J * TS) + 16 * q);
                cp_async16(st + TS * sizeof(T) + 16 * q, (const char *)(gE + tb + (size_t)J * TS) + 16 * q);
                if (hasZ)
                    cp_async16(st + 2 * TS * sizeof(T) + 16 * q, (const char *)(gX + tb + (size_t)J * TS) + 16 * q);
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int i = 0; i < D - 1; i++) issue(i);
    T x = gX[tb + (size_t)M * TS + cm]; // X_M (column-major)
    for (int i = 0; i < cnt; i++) {
        const int J = blk(i);
        issue(i + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
        const T *sc = slot + (i % D) * C::STAGE;
        T t = hasZ ? sc[2 * TS + rm] : sc_zero<T>(); // Z_J (row-major)
        const T ev = sc[TS + cm], gv = sc[cm];     // the coupling tile and G_J or H_J (column-major)
        __syncwarp(m); // the ring entry may be refilled from here on
        t = el_msub<T, KB>(m, t, ev, x, r, c);
        x = el_mul<T, KB>(m, gv, t, r, c);
        gX[tb + (size_t)J * TS + cm] = x;
    }
    cp_async_wait_all();
}

// Partitions [part0, part1): the forward part (both elimination chains, the
// spikes' forward sweeps, the middle block) or the back substitution.
template <class T, int KB> int run_twist(spk_plan *P, cudaStream_t st, bool fwd, int part0, int part1)
{
    if constexpr (!TwistFits<T, KB>::ok) {
        return SPK_EBAND;
    } else {
        using C = TwistFits<T, KB>;
        constexpr int NT = TwCfg<T, KB>::NT_PROD, NT_LU = TwCfg<T, KB>::NT_LU;
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(k_tw_lu<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_tw_sweep<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_tw_merge<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_tw_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::smem) !=
                    cudaSuccess)
                return SPK_ECUDA;
            if constexpr (tw_lu_w_ok<T, KB>()) {
                if (cudaFuncSetAttribute(k_tw_lu_w<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tw_lu_w_smem<T, KB>()) != cudaSuccess ||
                    cudaFuncSetAttribute(k_tw_bwd_w<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tw_lu_w_smem<T, KB>()) != cudaSuccess ||
                    cudaFuncSetAttribute(k_tw_sweep_w<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tw_sweep_w_smem<T, KB>()) != cudaSuccess)
                    return SPK_ECUDA;
            }
            attr = true;
        }
        const int p = P->p, np = part1 - part0;
        if (np <= 0) return SPK_OK;
        if (fwd) {
            if constexpr (tw_lu_w_ok<T, KB>())
                k_tw_lu_w<T, KB><<<(2 * np + TW_W_CHAINS - 1) / TW_W_CHAINS, 32 * TW_W_CHAINS,
                                   tw_lu_w_smem<T, KB>(), st>>>((const T *)P->d_T, P->d_blk_off, (T *)P->d_L,
                                                                (T *)P->d_G, (T *)P->d_E, P->d_err, part0, np);
            else
                k_tw_lu<T, KB><<<dim3(np, 2), NT_LU, C::smem, st>>>((const T *)P->d_T, P->d_blk_off, (T *)P->d_L,
                                                                    (T *)P->d_G, (T *)P->d_E, P->d_err, part0);
            SPK_CHECK_LAUNCH();
            P->launches++;
            if (p > 1) {
                if constexpr (tw_lu_w_ok<T, KB>())
                    k_tw_sweep_w<T, KB><<<(2 * np + TW_W_CHAINS - 1) / TW_W_CHAINS, 32 * TW_W_CHAINS,
                                          tw_sweep_w_smem<T, KB>(), st>>>(
                        P->d_part_start, P->d_blk_off, p, (const T *)P->d_L, (const T *)P->d_E,
                        (const T *)P->d_Bhat, (T *)P->d_V, (T *)P->d_W, part0, np, P->d_err);
                else
                    k_tw_sweep<T, KB><<<dim3(np, 2), NT, C::smem, st>>>(P->d_part_start, P->d_blk_off, p,
                                                                        (const T *)P->d_L, (const T *)P->d_E,
                                                                        (const T *)P->d_Bhat, (T *)P->d_V,
                                                                        (T *)P->d_W, part0, P->d_err);
                SPK_CHECK_LAUNCH();
                P->launches++;
            }
            k_tw_merge<T, KB><<<np, NT_LU, C::smem, st>>>((const T *)P->d_T, P->d_blk_off, p, (T *)P->d_L,
                                                                    (T *)P->d_G, (T *)P->d_V, (T *)P->d_W, P->d_err,
                                                                    part0);
            SPK_CHECK_LAUNCH();
            P->launches++;
        } else if (p > 1) {
            if constexpr (tw_lu_w_ok<T, KB>())
                k_tw_bwd_w<T, KB><<<(4 * np + TW_W_CHAINS - 1) / TW_W_CHAINS, 32 * TW_W_CHAINS,
                                    tw_lu_w_smem<T, KB>(), st>>>(P->d_blk_off, p, (const T *)P->d_G,
                                                                 (const T *)P->d_E, (T *)P->d_V, (T *)P->d_W, part0,
                                                                 np, P->d_err);
            else
                k_tw_bwd<T, KB><<<dim3(np, 4), NT, C::smem, st>>>(P->d_blk_off, p, (const T *)P->d_G,
                                                                  (const T *)P->d_E, (T *)P->d_V, (T *)P->d_W, part0,
                                                                  P->d_err);
            SPK_CHECK_LAUNCH();
            P->launches++;
        }
        return SPK_OK;
    }
}

template <class T, int KB> int run_qtwist(spk_plan *P, cudaStream_t st, bool fwd, int part0, int part1)
{
    using C = QTw<T, KB>;
    if (part0 != 0 || part1 != P->p) return SPK_EARG; // whole plans only
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_qtw_lu<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_qtw_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM) !=
                cudaSuccess)
            return SPK_ECUDA;
        attr = true;
    }
    const int p = P->p;
    if (fwd) {
        const int cpc = chains_per_cta(2LL * p, C::CPC);
        k_qtw_lu<T, KB><<<2 * ((p + cpc - 1) / cpc), cpc * C::EL, (size_t)cpc * C::SLOT, st>>>(
            (const T *)P->d_T, P->d_part_start, P->d_blk_off, p, (const T *)P->d_Bhat, (T *)P->d_L, (T *)P->d_G,
            (T *)P->d_E, (T *)P->d_V, (T *)P->d_W, P->d_err);
        SPK_CHECK_LAUNCH();
        const int mpc = 32; // chains per CTA of the middle-block kernel
        k_qtw_merge<T, KB><<<(p + mpc - 1) / mpc, mpc * KB, 0, st>>>((const T *)P->d_T, P->d_blk_off, p, (T *)P->d_L,
                                                                     (T *)P->d_G, (T *)P->d_V, (T *)P->d_W, P->d_err);
        SPK_CHECK_LAUNCH();
        P->launches += 2;
    } else if (p > 1) {
        const int cpc = chains_per_cta(4LL * p, C::CPC);
        k_qtw_bwd<T, KB><<<(4 * p + cpc - 1) / cpc, cpc * C::EL, (size_t)cpc * C::SLOT, st>>>(
            P->d_blk_off, p, (const T *)P->d_G, (const T *)P->d_E, (T *)P->d_V, (T *)P->d_W);
        SPK_CHECK_LAUNCH();
        P->launches++;
    }
    return SPK_OK;
}

template <class T> int disp_twist(spk_plan *P, cudaStream_t st, bool fwd, int part0, int part1)
{
    switch (P->KB) {
    case 2: return run_qtwist<T, 2>(P, st, fwd, part0, part1);
    case 4: return run_qtwist<T, 4>(P, st, fwd, part0, part1);
    case 16: return run_twist<T, 16>(P, st, fwd, part0, part1);
    case 32: return run_twist<T, 32>(P, st, fwd, part0, part1);
    case 64: return run_twist<T, 64>(P, st, fwd, part0, part1);
    default: return SPK_EBAND;
    }
}

template <class T> bool twist_ok(int KB)
{
    switch (KB) {
    case 2:
    case 4: return true; // KB lanes per chain: no shared-memory tiles to fit
    case 16: return TwistFits<T, 16>::ok;
    case 32: return TwistFits<T, 32>::ok;
    case 64: return TwistFits<T, 64>::ok;
    default: return false;
    }
}

} // namespace

extern "C" int spk_twist_supported(int KB, int is_complex, int mode)
{
    if (is_complex) return mode == SPK_MIXED ? twist_ok<cfloat>(KB) : twist_ok<cdouble>(KB);
    return mode == SPK_MIXED ? twist_ok<float>(KB) : twist_ok<double>(KB);
}

extern "C" int spk_twist_factor(spk_plan *P, int forward, int part0, int part1, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    const bool f = forward != 0;
    if (P->is_complex)
        return P->mode == SPK_MIXED ? disp_twist<cfloat>(P, st, f, part0, part1)
                                    : disp_twist<cdouble>(P, st, f, part0, part1);
    return P->mode == SPK_MIXED ? disp_twist<float>(P, st, f, part0, part1) : disp_twist<double>(P, st, f, part0, part1);
}
