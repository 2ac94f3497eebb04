// spike_factor.cu -- factorization phase of the SPIKE solve on sm_103a.
//
// Replaces the reference's factorization loop (OpenMP/spike_interfaces.c
// :105-237): per partition it extracted A_i as CSR (matrix_ExtractMatrix,
// OpenMP/spike_matrix.c:563), factored it with SuperLU (OpenMP/
// spike_superlu.c:763), extracted dense B_i / C_i (matrix_ExtractBlock,
// OpenMP/spike_matrix.c:421) and solved A_i V_i = B_i, A_i W_i = C_i column by
// column, then scattered the tips into R (OpenMP/spike_matrix.c:1414).
//
// Here one CTA owns one partition and walks it as a block-tridiagonal matrix
// with KB x KB blocks (KB >= max(ku, kl)); the CSR is read exactly once:
//
//   k_band_tiles   (K1) CSR rows of every block -> dense factor-precision tiles
//                  D_J, F_{J-1}^T, E_J, C^, B^; one CTA per block, in parallel.
//   k_factor_fwd   (K2) L_J = F_{J-1} G_{J-1},  S_J = D_J - L_J E_{J-1},
//                  G_J = S_J^{-1} (Gauss-Jordan), and the forward sweep of the
//                  W spike z_J = -L_J z_{J-1} (z_0 = C^_i).  Stores L, G, z.
//   k_factor_bwd   (K3) backward sweep X_J = G_J (Z_J - E_J X_{J+1}) for
//                  [V | W] (V's right-hand side B^_i lives in the last rows
//                  only), storing the full spikes for explicit retrieval.
//   k_tips         bottom/top tips of V and W into the FP64 interface blocks
//                  of the reduced system.
//
// Pivot-free: A is required to be diagonally dominant enough that block
// elimination needs no pivoting (every shipped workload is).  A zero or
// non-finite pivot sets SPK_DEV_ERR_PIVOT and the host returns SPIKE_ERROR.
#include "spike_common.cuh"

#include <type_traits>

namespace {

template <class T, int KB> struct FactorSmem {
    using TL = Tile<T, KB, NTOf<KB>::value>;
    // 128-row tiles (FP32 only): three resident tiles per CTA, see k_factor_fwd_big
    static constexpr bool BIG = KB >= 128;
    static constexpr size_t tile = sizeof(T) * TL::ELEMS;
    static constexpr size_t fwd = (BIG ? 3 : 6) * tile + sizeof(T) * TL::INV_BUF + 64;
    // k_band_tiles: small tiles pack BG row blocks into one CTA (one warp or
    // warp pair each), so the grid is not a million one-warp CTAs
    static constexpr int BG = KB <= 16 ? 256 / NTOf<KB>::value : 1;
    static constexpr size_t band_one = (3 * sizeof(T) * KB * (KB + 1) + sizeof(int) * (KB + 1) + 15) / 16 * 16;
    static constexpr size_t band = BG * band_one + 64;
    static constexpr size_t bwd = (BIG ? 3 : 6) * tile + 64; // (also k_wsweep_big: three tiles)
};

// Scatter the CSR rows of block J of partition [s, e) into the shared tiles.
// F: columns of block J-1 (stored transposed: it is the left operand of
// F G), D: block J, En: block J+1 (shared tiles, row stride LD); gZ (global,
// row-major, zeroed by the caller): C^ coupling (J == 0, columns s-KB..s-1);
// gBhat (global, row-major): B^ coupling (columns e..e+KB-1).
// One warp per row: the row's entries are contiguous, so the loads are
// coalesced and every entry's row is known without a search; up to five
// 32-entry chunks of a row (a whole row of a 64-row tile's band) are in
// flight per iteration.
template <class T, class H, int KB, int LD>
__device__ __forceinline__ void place_entry(int lr, int lrow, int c, H a, int s, int m, int J, T *F, T *D, T *En,
                                            T *gZ, T *gBhat, unsigned *err)
{
    const T v = cvt_fast<T, H>(a);
    const int lc = c - s;
    if (lc < 0) {
        const int cc = lc + KB;
        if (cc >= 0 && lrow < KB) {
            if (gZ) gZ[lr * KB + cc] = v;
        } else
            atomicOr(err, SPK_DEV_ERR_BAND);
    } else if (lc >= m) {
        const int br = lrow - (m - KB), bc = lc - m;
        if (br >= 0 && bc < KB) {
            if (gBhat) gBhat[br * KB + bc] = v;
        } else
            atomicOr(err, SPK_DEV_ERR_BAND);
    } else {
        const int bc = lc / KB, cc = lc - bc * KB;
        const int d = bc - J;
        if (d == 0)
            D[lr * LD + cc] = v;
        else if (d == -1)
            F[cc * LD + lr] = v;
        else if (d == 1)
            En[lr * LD + cc] = v;
        else
            atomicOr(err, SPK_DEV_ERR_BAND);
    }
}

// VAL: the single-system path skipped its separate analysis pass (the plan
// was reused), so this pass also validates the CSR -- row pointers in range
// and non-decreasing, columns in [0, n) and increasing within a row -- and
// measures the exact bandwidth: err[1] = ku, err[2] = kl.  A row with bad
// pointers is flagged and not read.  impl_kl >= 0: colind is not read; the
// host verified that every row is the full band, so entry t of row r is
// column max(0, r - impl_kl) + (t - rowptr[r]).
template <class T, class H, int KB, int LD, bool VAL, bool IMPL = false>
__device__ __forceinline__ void scatter_block(const int *__restrict__ rowptr, const int *__restrict__ colind,
                              const H *__restrict__ aij, int s, int e, int J, T *F, T *D, T *En, T *gZ,
                              T *gBhat, unsigned *err, int *srp, int n, long long nnz, int impl_kl, int tid,
                              bool live)
{
    constexpr int NT = NTOf<KB>::value;
    constexpr int NW = NT / 32;
    const int m = e - s;
    const int lrow0 = J * KB;
    const int nr = min(KB, m - lrow0); // real rows in the block, >= 1
    if (live) {
        for (int q = tid; q <= nr; q += NT) srp[q] = rowptr[s + lrow0 + q];
        for (int lr = nr + tid; lr < KB; lr += NT) D[lr * LD + lr] = sc_one<T>(); // identity padding
    }
    __syncthreads();
    if (!live) return; // (a CTA's spare block slot: every barrier above is shared)
    const int warp = tid >> 5, lane = tid & 31;
    // pieces per iteration: a whole row of the band (2 KB + 1 entries) in one go
    constexpr int PPR = (2 * KB + 1 + 31) / 32 < 1 ? 1 : (2 * KB + 1 + 31) / 32 > 5 ? 5 : (2 * KB + 1 + 31) / 32;
    int ku = 0, kl = 0;
    if constexpr (KB <= 16) {
        // Short rows (2 KB + 1 <= 33 entries): the block's entries are one
        // contiguous run, so the threads take it flat -- every entry of every
        // row in flight at once -- and find each entry's row among the block's
        // row pointers in shared memory.
        const int T0 = srp[0], T1 = srp[nr];
        bool rows_ok = T0 >= 0 && (long long)T1 <= nnz && T1 >= T0;
        if constexpr (VAL) {
            for (int q = tid; q < nr; q += NT)
                if (srp[q] < 0 || (long long)srp[q + 1] > nnz || srp[q + 1] < srp[q]) atomicOr(err, SPK_DEV_ERR_CSR);
            if (!rows_ok && tid == 0) atomicOr(err, SPK_DEV_ERR_CSR);
        }
        constexpr int U = 4; // entries per thread in flight
        for (int base = rows_ok ? T0 : T1; base < T1; base += NT * U) {
            int c[U], lrs[U];
            H a[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int t = base + tid + u * NT;
                lrs[u] = 0;
                if (t < T1) {
                    int lr = 0;
#pragma unroll
                    for (int q = 1; q < KB; q++) lr += (q < nr && srp[q] <= t);
                    lrs[u] = lr;
                    c[u] = IMPL ? max(0, s + lrow0 + lr - impl_kl) + (t - srp[lr]) : __ldg(colind + t);
                    a[u] = aij[t];
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int t = base + tid + u * NT;
                if (t < T1) {
                    const int lr = lrs[u], grow = s + lrow0 + lr;
                    if constexpr (VAL) {
                        if (c[u] < 0 || c[u] >= n || (t > srp[lr] && __ldg(colind + t - 1) >= c[u]))
                            atomicOr(err, SPK_DEV_ERR_CSR);
                        ku = max(ku, c[u] - grow);
                        kl = max(kl, grow - c[u]);
                    }
                    place_entry<T, H, KB, LD>(lr, lrow0 + lr, c[u], a[u], s, m, J, F, D, En, gZ, gBhat, err);
                }
            }
        }
    } else
    for (int lr = warp; lr < nr; lr += NW) {
        const int t0 = srp[lr], t1 = srp[lr + 1];
        if (VAL && (t0 < 0 || (long long)t1 > nnz || t1 < t0)) {
            if (lane == 0) atomicOr(err, SPK_DEV_ERR_CSR);
            continue;
        }
        const int grow = s + lrow0 + lr; // the row's index in the system
        const int cfirst = IMPL ? max(0, grow - impl_kl) - t0 : 0; // implied columns: cfirst + t
        int carry = -1;                  // last column of the previous iteration
        for (int base = t0; base < t1; base += 32 * PPR) { // warp-uniform: the shuffles see every lane
            const int t = base + lane;
            int c[PPR];
            H a[PPR];
#pragma unroll
            for (int u = 0; u < PPR; u++) // the row's 32-entry pieces in flight at once
                if (t + 32 * u < t1) {
                    c[u] = IMPL ? cfirst + t + 32 * u : __ldg(colind + t + 32 * u);
                    a[u] = aij[t + 32 * u];
                }
            if constexpr (VAL) {
#pragma unroll
                for (int u = 0; u < PPR; u++) {
                    const int up = __shfl_up_sync(0xffffffffu, c[u], 1);
                    const int wrap = __shfl_sync(0xffffffffu, u ? c[u > 0 ? u - 1 : 0] : carry, 31);
                    const int pred = lane ? up : (u ? wrap : carry);
                    const int tt = t + 32 * u;
                    if (tt < t1) {
                        if (c[u] < 0 || c[u] >= n || (tt > t0 && pred >= c[u])) atomicOr(err, SPK_DEV_ERR_CSR);
                        ku = max(ku, c[u] - grow);
                        kl = max(kl, grow - c[u]);
                    }
                }
                carry = __shfl_sync(0xffffffffu, c[PPR - 1], 31); // used only when the next iteration's entries exist
            }
#pragma unroll
            for (int u = 0; u < PPR; u++)
                if (t + 32 * u < t1)
                    place_entry<T, H, KB, LD>(lr, lrow0 + lr, c[u], a[u], s, m, J, F, D, En, gZ, gBhat, err);
        }
    }
    if constexpr (VAL) {
        for (int o = 16; o > 0; o >>= 1) {
            ku = max(ku, __shfl_xor_sync(0xffffffffu, ku, o));
            kl = max(kl, __shfl_xor_sync(0xffffffffu, kl, o));
        }
        // every warp of every block reaches here: read first and update only
        // with a larger value, so the two words see a handful of atomics
        // instead of millions serialised at one L2 slice (a stale read only
        // costs an atomic that was not needed)
        if (lane == 0) {
            if ((unsigned)ku > *(volatile const unsigned *)(err + 1)) atomicMax(err + 1, (unsigned)ku);
            if ((unsigned)kl > *(volatile const unsigned *)(err + 2)) atomicMax(err + 2, (unsigned)kl);
        }
    }
}

template <class T, int KB, int LD = TileLD<T, KB>::value> __device__ __forceinline__ void zero_tile(T *s)
{
    constexpr int NT = NTOf<KB>::value;
    for (int q = threadIdx.x; q < KB * LD; q += NT) s[q] = sc_zero<T>();
}

// shared tile -> dense global tile (row-major)
template <class T, int KB, int LD = TileLD<T, KB>::value> __device__ __forceinline__ void store_tile(T *g, const T *s)
{
    constexpr int NT = NTOf<KB>::value;
    for (int q = threadIdx.x; q < KB * KB; q += NT) {
        const int r = q / KB, c = q - r * KB;
        g[q] = s[r * LD + c];
    }
}
// dense global tile (row-major) -> shared tile
template <class T, int KB> __device__ __forceinline__ void load_tile(T *s, const T *g)
{
    copy_tile_g2s<T, KB, NTOf<KB>::value>(s, g);
}
// shared tile -> global tile, column-major (retrieval reads of V / W; factor
// tiles that later serve as left operands)
template <class T, int KB, int LD = TileLD<T, KB>::value>
__device__ __forceinline__ void store_tile_cm(T *g, const T *s)
{
    constexpr int NT = NTOf<KB>::value;
    for (int q = threadIdx.x; q < KB * KB; q += NT) {
        const int c = q / KB, r = q - c * KB;
        g[q] = s[r * LD + c];
    }
}

// K1: one CTA per row block (all partitions at once, fully parallel).  Reads
// the block's CSR rows once and writes, in factor precision, the tiles the
// sequential chain consumes: D_J (row-major), F_{J-1}^T and E_J (row-major)
// into gT, E_J column-major into gE for the backward sweep, C^ into the W
// spike's first tile (J == 0) and B^ into gBhat (last rows).  With twist set,
// blocks past the partition's middle block M = N/2 are stored for the
// bottom-up chain instead (spike_twist.cu): A(J,J-1) row-major in gT and
// column-major in gE for J > M, A(J,J+1) column-major in gT for J >= M.
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value * FactorSmem<T, KB>::BG)
    k_band_tiles(const int *__restrict__ rowptr, const int *__restrict__ colind,
                 const typename HighOf<T>::type *__restrict__ aij, const int *__restrict__ part_start,
                 const int *__restrict__ blk_off, const int *__restrict__ blk_part, T *gT, T *gE, T *gZ, T *gBhat,
                 unsigned *err, const spk_sysref *__restrict__ sys, const int *__restrict__ part_sys, int twist,
                 int validate, int n, long long nnz, int gb0, int gb_end, int nb_total, int impl_kl)
{
    using H = typename HighOf<T>::type;
    using FS = FactorSmem<T, KB>;
    constexpr int NT = NTOf<KB>::value;
    constexpr size_t TS = (size_t)KB * KB;
    // this launch covers blocks [gb0, gb_end), FS::BG per CTA (NT threads each)
    const int grp = threadIdx.x / NT, tid = threadIdx.x - grp * NT;
    const int gb = (int)blockIdx.x * FS::BG + grp + gb0;
    const bool live = gb < gb_end;
    const int part = live ? blk_part[gb] : 0;
    const int J = live ? gb - blk_off[part] : 0;
    const int M = twist && live ? (blk_off[part + 1] - blk_off[part]) / 2 : 1 << 30; // middle block
    int s = live ? part_start[part] : 0, e = live ? part_start[part + 1] : 0;
    const bool zt = live && J == 0 && part > 0;
    if (sys && live) { // batch group: the partition's own system, in its local rows
        const spk_sysref &S = sys[part_sys[part]];
        rowptr = S.rowptr;
        colind = S.colind;
        aij = (const H *)S.aij;
        s -= (int)S.row0;
        e -= (int)S.row0;
    }

    // odd row stride: conflict-free for the row-major and the column-major stores
    constexpr int LD1 = KB + 1;
    constexpr int EL1 = KB * LD1;
    extern __shared__ char smraw[];
    T *sD = (T *)(smem_align(smraw) + grp * FS::band_one), *sF = sD + EL1, *sE = sF + EL1;
    int *srp = (int *)(sE + EL1);
    T *gz = zt ? gZ + (size_t)blk_off[part] * TS : nullptr;
    for (int q = tid; q < 3 * EL1; q += NT) sD[q] = sc_zero<T>(); // sD, sF, sE are consecutive
    if (zt)
        for (int q = tid; q < KB * KB; q += NT) gz[q] = sc_zero<T>();
    __syncthreads();
    if (validate) {
        scatter_block<T, H, KB, LD1, true>(rowptr, colind, aij, s, e, J, sF, sD, sE, gz, gBhat + (size_t)part * TS,
                                           err, srp, n, nnz, impl_kl, tid, live);
        if (live && tid == 0 && ((gb == 0 && rowptr[0] != 0) || (gb == nb_total - 1 && (long long)rowptr[n] != nnz)))
            atomicOr(err, SPK_DEV_ERR_CSR);
    } else if (impl_kl >= 0) {
        scatter_block<T, H, KB, LD1, false, true>(rowptr, colind, aij, s, e, J, sF, sD, sE, gz,
                                                  gBhat + (size_t)part * TS, err, srp, n, nnz, impl_kl, tid, live);
    } else {
        scatter_block<T, H, KB, LD1, false>(rowptr, colind, aij, s, e, J, sF, sD, sE, gz, gBhat + (size_t)part * TS,
                                            err, srp, n, nnz, impl_kl, tid, live);
    }
    __syncthreads();
    if (!live) return;
    // shared tile (row stride LD1) -> global tile, row-major or column-major
    auto put = [&](T *g, const T *sm, bool cm) {
        for (int q = tid; q < KB * KB; q += NT) {
            const int a = q / KB, b = q - a * KB;
            g[q] = cm ? sm[b * LD1 + a] : sm[a * LD1 + b];
        }
    };
    T *g = gT + (size_t)gb * 3 * TS;
    put(g, sD, false);
    put(g + TS, sF, J > M); // J <= M: the shared image of F^T, A(J,J-1) column-major; beyond: row-major
    if (J < M) {
        put(g + 2 * TS, sE, false);
        put(gE + (size_t)gb * TS, sE, true);
    } else {
        put(g + 2 * TS, sE, true); // A(J,J+1) column-major
        if (J > M) put(gE + (size_t)gb * TS, sF, false); // A(J,J-1) column-major
    }
}

// K1 for tiles of up to 4 rows: one thread per padded row, one warp per 32
// consecutive rows (32 / KB blocks).  A block of such tiles holds a few dozen
// entries, so a CTA per block group spends its time on dependent memory round
// trips; here every row's entries are in flight at once.  Each row goes into
// the warp's copy of its blocks' tiles in shared memory (zeros, the identity
// on D's diagonal for a padding row, then its entries), and the warp writes
// the tiles out with coalesced stores: a row written straight to global
// memory would touch every 32-byte sector of its tiles once per column, and
// those partial-sector writes, not DRAM, set the time.  The C^ and B^
// coupling tiles (one block per partition) are still written per row.  The
// tiles, layouts, couplings, validation and bandwidth are those of
// k_band_tiles.
constexpr int BAND_ROWS_WARPS = 4; // warps per CTA

template <class T, int KB>
__global__ void __launch_bounds__(32 * BAND_ROWS_WARPS)
    k_band_rows(const int *__restrict__ rowptr, const int *__restrict__ colind,
                const typename HighOf<T>::type *__restrict__ aij, const int *__restrict__ part_start,
                const int *__restrict__ blk_off, const int *__restrict__ blk_part, T *gT, T *gE, T *gZ, T *gBhat,
                unsigned *err, const spk_sysref *__restrict__ sys, const int *__restrict__ part_sys, int twist,
                int validate, int n, long long nnz, int gb0, int gb_end, int nb_total, int impl_kl)
{
    using H = typename HighOf<T>::type;
    constexpr int TS = KB * KB;
    constexpr int BW = 32 / KB;      // blocks per warp pass
    constexpr int ST = 3 * TS + 1;   // shared stride of a block's (D, slot 1, slot 2); +1 spreads the banks
    constexpr int SE = TS + 1;       // shared stride of a block's column-major coupling tile for gE
    __shared__ T stage[BAND_ROWS_WARPS][BW * (ST + SE)];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    T *sT = stage[wib], *sE = sT + BW * ST;
    const int bw = lane / KB, lr = lane - bw * KB; // this lane's block in the pass and row in the block
    int ku = 0, kl = 0;
    bool bad_csr = false, bad_band = false;
    const long long r0 = (long long)gb0 * KB, r1 = (long long)gb_end * KB;
    const long long wstride = (long long)gridDim.x * BAND_ROWS_WARPS * 32;
    // warp-uniform passes: every lane runs every pass (the shuffles and
    // __syncwarp below need the whole warp)
    for (long long wb = r0 + ((long long)blockIdx.x * BAND_ROWS_WARPS + wib) * 32; wb < r1; wb += wstride) {
        const int gbw = (int)(wb / KB); // first block of the pass (wb is a multiple of KB)
        const int nb = (int)min((long long)BW, (long long)gb_end - gbw);
        for (int q = lane; q < BW * (ST + SE); q += 32) sT[q] = sc_zero<T>(); // sT and sE are consecutive
        __syncwarp();
        const int gb = gbw + bw;
        const bool act = bw < nb;
        int write_e = 0; // gE is written for every block but the middle one
        if (act) {
            const int part = blk_part[gb];
            const int J = gb - blk_off[part];
            const int M = twist ? (blk_off[part + 1] - blk_off[part]) / 2 : 1 << 30; // middle block
            write_e = J != M;
            int s = part_start[part], e = part_start[part + 1];
            const int *rp = rowptr, *ci = colind;
            const H *av = aij;
            if (sys) { // batch group: the partition's own system, in its local rows
                const spk_sysref &S = sys[part_sys[part]];
                rp = S.rowptr;
                ci = S.colind;
                av = (const H *)S.aij;
                s -= (int)S.row0;
                e -= (int)S.row0;
            }
            const int m = e - s, lrow = J * KB + lr;
            T *tD = sT + bw * ST, *t1 = tD + TS, *t2 = tD + 2 * TS, *tE = sE + bw * SE;
            const bool cm1 = J <= M; // A(J,J-1) in slot 1: column-major up to the middle block
            const bool cm2 = J >= M; // A(J,J+1) in slot 2: column-major from the middle block on
            T *gz = (J == 0 && part > 0) ? gZ + (size_t)blk_off[part] * TS : nullptr; // C^ (W's first tile)
            auto put = [&](T *t, int c, bool cm, T v) { (cm ? t[c * KB + lr] : t[lr * KB + c]) = v; };
            if (gz)
#pragma unroll
                for (int c = 0; c < KB; c++) gz[lr * KB + c] = sc_zero<T>();
            if (validate && lr == 0 && ((gb == 0 && rowptr[0] != 0) || (gb == nb_total - 1 && (long long)rowptr[n] != nnz)))
                bad_csr = true;
            const int grow = s + lrow;
            const int t0 = lrow < m ? rp[grow] : 0, t1e = lrow < m ? rp[grow + 1] : 0;
            if (lrow >= m) {
                tD[lr * KB + lr] = sc_one<T>(); // identity padding row
            } else if (t0 < 0 || t1e < t0 || (long long)t1e > nnz) { // a row that cannot be read
                if (validate) bad_csr = true;
            } else {
                const int cfirst = impl_kl >= 0 ? max(0, grow - impl_kl) - t0 : 0; // implied columns: cfirst + t
                for (int t = t0; t < t1e; t++) {
                    const int c = impl_kl >= 0 ? cfirst + t : __ldg(ci + t);
                    const T v = cvt_fast<T, H>(av[t]);
                    if (validate) {
                        if (c < 0 || c >= n || (t > t0 && __ldg(ci + t - 1) >= c)) bad_csr = true;
                        ku = max(ku, c - grow);
                        kl = max(kl, grow - c);
                    }
                    const int lc = c - s;
                    if (lc < 0) {
                        const int cc = lc + KB;
                        if (cc >= 0 && lrow < KB) {
                            if (gz) gz[lr * KB + cc] = v;
                        } else
                            bad_band = true;
                    } else if (lc >= m) {
                        const int br = lrow - (m - KB), bc = lc - m;
                        if (br >= 0 && bc < KB)
                            gBhat[(size_t)part * TS + br * KB + bc] = v;
                        else
                            bad_band = true;
                    } else {
                        const int bc = lc / KB, cc = lc - bc * KB, d = bc - J;
                        if (d == 0) {
                            put(tD, cc, false, v);
                        } else if (d == -1) {
                            put(t1, cc, cm1, v);
                            if (J > M) put(tE, cc, true, v); // A(J,J-1) column-major for the bottom chain
                        } else if (d == 1) {
                            put(t2, cc, cm2, v);
                            if (J < M) put(tE, cc, true, v); // A(J,J+1) column-major for the top chain
                        } else {
                            bad_band = true;
                        }
                    }
                }
            }
        }
        __syncwarp();
        // the pass's tiles out: (D, slot 1, slot 2) of its blocks are one
        // contiguous run of gT, their gE tiles one run of gE
        T *oT = gT + (size_t)gbw * 3 * TS;
        for (int q = lane; q < nb * 3 * TS; q += 32) {
            const int b = q / (3 * TS);
            oT[q] = sT[b * ST + (q - b * 3 * TS)];
        }
        T *oE = gE + (size_t)gbw * TS;
        for (int q0 = 0; q0 < BW * TS; q0 += 32) {
            const int q = q0 + lane, b = q / TS < BW ? q / TS : BW - 1;
            const int we = __shfl_sync(0xffffffffu, write_e, b * KB);
            if (q < nb * TS && we) oE[q] = sE[b * SE + (q - b * TS)];
        }
        __syncwarp(); // the next pass zeroes the staging tiles
    }
    if (bad_csr) atomicOr(err, SPK_DEV_ERR_CSR);
    if (bad_band) atomicOr(err, SPK_DEV_ERR_BAND);
    if (validate) {
        for (int o = 16; o > 0; o >>= 1) {
            ku = max(ku, __shfl_xor_sync(0xffffffffu, ku, o));
            kl = max(kl, __shfl_xor_sync(0xffffffffu, kl, o));
        }
        if ((threadIdx.x & 31) == 0) {
            if ((unsigned)ku > *(volatile const unsigned *)(err + 1)) atomicMax(err + 1, (unsigned)ku);
            if ((unsigned)kl > *(volatile const unsigned *)(err + 2)) atomicMax(err + 2, (unsigned)kl);
        }
    }
}

// K1 over row blocks [b0, b1) of the plan: k_band_rows for tiles of up to 4
// rows (at 4-row complex tiles and 4 million rows 0.27 ms, against 0.56 ms
// with each row written straight to global memory and 0.78 ms for
// k_band_tiles), k_band_tiles above
template <class T, int KB>
int launch_band_tiles(spk_plan *P, const int *rowptr, const int *colind, const void *aij, int b0, int b1,
                      cudaStream_t st)
{
    using H = typename HighOf<T>::type;
    using S = FactorSmem<T, KB>;
    constexpr int NT = NTOf<KB>::value;
    const int val = P->validate && !P->d_sys && !P->impl_cols;
    const int ikl = P->impl_cols ? P->impl_kl : -1;
    if constexpr (KB <= 4) {
        const long long rows = (long long)(b1 - b0) * KB, per = 32LL * BAND_ROWS_WARPS;
        const long long g = (rows + per - 1) / per < 152LL * 16 ? (rows + per - 1) / per : 152LL * 16;
        const int grid = (int)g;
        k_band_rows<T, KB><<<grid > 0 ? grid : 1, 32 * BAND_ROWS_WARPS, 0, st>>>(
            rowptr, colind, (const H *)aij, P->d_part_start, P->d_blk_off, P->d_blk_part, (T *)P->d_T, (T *)P->d_E,
            (T *)P->d_W, (T *)P->d_Bhat, P->d_err, P->d_sys, P->d_part_sys, P->twist, val, P->n, P->nnz, b0, b1,
            P->total_blocks, ikl);
    } else {
        k_band_tiles<T, KB><<<(b1 - b0 + S::BG - 1) / S::BG, NT * S::BG, S::band, st>>>(
            rowptr, colind, (const H *)aij, P->d_part_start, P->d_blk_off, P->d_blk_part, (T *)P->d_T, (T *)P->d_E,
            (T *)P->d_W, (T *)P->d_Bhat, P->d_err, P->d_sys, P->d_part_sys, P->twist, val, P->n, P->nnz, b0, b1,
            P->total_blocks, ikl);
    }
    SPK_CHECK_LAUNCH();
    return SPK_OK;
}

// K2: the sequential block-LU chain of one partition per CTA.
//   L_J = F_{J-1} G_{J-1},  S_J = D_J - L_J E_{J-1},  G_J = S_J^{-1},
//   W forward sweep z_J = -L_J z_{J-1} (z_0 = C^).
// While G_J is being inverted, the tiles of block J+1 stream from gT into the
// three shared buffers that block J no longer reads (cp.async), so the chain
// never waits on memory.
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_factor_fwd(const T *__restrict__ gT, const int *__restrict__ blk_off, T *gL, T *gG, T *gZ, unsigned *err)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * 3 * TS;
    const bool doW = part > 0;

    extern __shared__ char smraw[];
    T *base = (T *)smem_align(smraw);
    T *sG = base, *sEp = sG + TL::ELEMS, *sEn = sEp + TL::ELEMS;
    T *sF = sEn + TL::ELEMS, *sD = sF + TL::ELEMS, *sZ = sD + TL::ELEMS;
    T *buf = sZ + TL::ELEMS;

    TL t(threadIdx.x);
    typename TL::Reg acc, accZ;
    bool ok = true;

    cp_async_tile<T, KB, NT>(sD, gTp);
    cp_async_tile<T, KB, NT>(sF, gTp + TS);
    cp_async_tile<T, KB, NT>(sEn, gTp + 2 * TS);
    if (doW) cp_async_tile<T, KB, NT>(sZ, gZ + tb); // z_0 = C^
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();

    for (int J = 0; J < N; J++) {
        if (J > 0) {
            // L_J = F_{J-1} G_{J-1}
            t.rzero(acc);
            t.mma_tu(acc, sF, sG); // F_{J-1} = A(J, J-1) is upper triangular (KB >= kl)
            __syncthreads();
            t.rstore_t(sF, acc); // sF now holds L_J, transposed
            t.gstore_t(gL + tb + J * TS, acc);
            __syncthreads();
            // S_J = D_J - L_J E_{J-1};  z_J = -L_J z_{J-1}
            t.rload(acc, sD);
            t.mms_t_bl(acc, sF, sEp); // E_{J-1} = A(J-1, J) is lower triangular
            if (doW) {
                t.rzero(accZ);
                t.mms_t(accZ, sF, sZ);
                __syncthreads();
                t.rstore(sZ, accZ);
                t.gstore(gZ + tb + J * TS, accZ);
            }
        } else {
            t.rload(acc, sD);
        }
        __syncthreads(); // sD, sF, sEp are free from here on
        if (J + 1 < N) {
            const T *gn = gTp + (size_t)(J + 1) * 3 * TS;
            cp_async_tile<T, KB, NT>(sD, gn);
            cp_async_tile<T, KB, NT>(sF, gn + TS);
            cp_async_tile<T, KB, NT>(sEp, gn + 2 * TS);
            cp_async_commit();
        }
        // G_J = S_J^{-1}
        ok = t.inverse(acc, buf) && ok;
        cp_async_wait_all();
        t.rstore(sG, acc);
        t.gstore_t(gG + tb + J * TS, acc); // column-major for the backward sweep
        T *tmp = sEp; // E_J becomes the previous block's coupling, E_{J+1} the current one
        sEp = sEn;
        sEn = tmp;
        __syncthreads();
    }
    if (!ok && threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

// Backward sweep for the spikes: X_J = G_J (Z_J - E_J X_{J+1}), X = [V | W].
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_factor_bwd(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                 const T *__restrict__ gL, const T *__restrict__ gG, const T *__restrict__ gE, T *gZ,
                 const T *__restrict__ gBhat, T *gV, T *gW)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int LD = TileLD<T, KB>::value;
    const int part = blockIdx.x;
    const int s = part_start[part], e = part_start[part + 1], m = e - s;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    const bool doW = part > 0, doV = part < p - 1;

    extern __shared__ char smraw[];
    T *base = (T *)smem_align(smraw);
    T *sG = base, *sE = sG + TL::ELEMS, *sZ = sE + TL::ELEMS, *sZV = sZ + TL::ELEMS;
    T *sXV = sZV + TL::ELEMS, *sXW = sXV + TL::ELEMS;

    TL t(threadIdx.x);
    typename TL::Reg aV, aW;

    // Forward sweep of V's right-hand side [0; B^]: nonzero only in the last
    // KB real rows, i.e. blocks J0 and J0+1 (when m is not a multiple of KB).
    const int J0 = (m - KB) / KB, o = (m - KB) - J0 * KB;
    if (doV) {
        // z_{J0}: rows o..KB-1 <- B^ rows 0..KB-1-o ; kept in gV tile J0 (row-major scratch)
        zero_tile<T, KB>(sZV);
        __syncthreads();
        for (int q = threadIdx.x; q < KB * KB; q += NT) {
            const int r = q / KB, c = q - r * KB;
            // (o < 0: a partition shorter than a tile takes B^'s last m rows)
            if (r >= o && r - o < KB) sZV[r * LD + c] = gBhat[(size_t)part * TS + (r - o) * KB + c];
        }
        __syncthreads();
        store_tile<T, KB>(gV + tb + J0 * TS, sZV);
        if (o > 0) {
            // z_{J0+1} = [B^ rows KB-o..KB-1 ; 0] - L_{J0+1} z_{J0}
            load_tile<T, KB>(sG, gL + tb + (J0 + 1) * TS);
            zero_tile<T, KB>(sZ);
            __syncthreads();
            for (int q = threadIdx.x; q < o * KB; q += NT) {
                const int r = q / KB, c = q - r * KB;
                sZ[r * LD + c] = gBhat[(size_t)part * TS + (KB - o + r) * KB + c];
            }
            __syncthreads();
            t.rload(aV, sZ);
            t.mms_t(aV, sG, sZV); // sG holds L_{J0+1} transposed
            __syncthreads();
            t.rstore(sZ, aV);
            __syncthreads();
            store_tile<T, KB>(gV + tb + (J0 + 1) * TS, sZ);
        }
        __syncthreads();
    }

    for (int J = N - 1; J >= 0; J--) {
        // all of the step's tiles in flight at once (one memory round trip)
        constexpr int NTC = NTOf<KB>::value;
        cp_async_tile<T, KB, NTC>(sG, gG + tb + J * TS);
        if (J < N - 1) cp_async_tile<T, KB, NTC>(sE, gE + tb + J * TS);
        if (doW) cp_async_tile<T, KB, NTC>(sZ, gZ + tb + J * TS);
        const bool hasZV = doV && (J == J0 || (o > 0 && J == J0 + 1));
        if (hasZV) cp_async_tile<T, KB, NTC>(sZV, gV + tb + J * TS);
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        // T = Z_J - E_J X_{J+1}
        if (doV) {
            if (hasZV)
                t.rload(aV, sZV);
            else
                t.rzero(aV);
            if (J < N - 1) t.mms_tl(aV, sE, sXV); // E_J = A(J, J+1) is lower triangular (KB >= ku)
        }
        if (doW) {
            t.rload(aW, sZ);
            if (J < N - 1) t.mms_tl(aW, sE, sXW);
        }
        __syncthreads();
        if (doV) t.rstore(sXV, aV);
        if (doW) t.rstore(sXW, aW);
        __syncthreads();
        // X_J = G_J T
        if (doV) {
            t.rzero(aV);
            t.mma_t(aV, sG, sXV);
        }
        if (doW) {
            t.rzero(aW);
            t.mma_t(aW, sG, sXW);
        }
        __syncthreads();
        if (doV) t.rstore(sXV, aV);
        if (doW) t.rstore(sXW, aW);
        __syncthreads();
        if (doV) store_tile_cm<T, KB>(gV + tb + J * TS, sXV);
        if (doW) store_tile_cm<T, KB>(gW + tb + J * TS, sXW);
        __syncthreads();
    }
}

// ------------------------------------------------------------ 128-row tiles
// A 128 x 128 FP32 tile takes 66 KB of shared memory, so a CTA (1024 threads,
// a 4 x 4 sub-tile each) keeps three of them resident instead of six: D_J
// goes from global memory straight into registers (its loads are issued
// before the L product and land during it), the W forward sweep runs as its
// own chain (k_wsweep_big) once the L tiles exist, and the backward sweep
// gives V and W a CTA each.  Same recurrences and global layouts as
// k_factor_fwd / k_factor_bwd.
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_factor_fwd_big(const T *__restrict__ gT, const int *__restrict__ blk_off, T *gL, T *gG, unsigned *err)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * 3 * TS; // per block: D, F^T, E (row-major)

    extern __shared__ char smraw[];
    T *sG = (T *)smem_align(smraw), *sE = sG + TL::ELEMS, *sF = sE + TL::ELEMS;
    T *buf = sF + TL::ELEMS;

    TL t(threadIdx.x);
    typename TL::Reg acc, dreg;
    bool ok = true;

    cp_async_tile<T, KB, NT>(sE, gTp + 2 * TS); // E_0
    if (N > 1) cp_async_tile<T, KB, NT>(sF, gTp + 3 * TS + TS);
    cp_async_commit();
    t.gload(acc, gTp); // S_0 = D_0
    for (int J = 0; J < N; J++) {
        if (J > 0) {
            t.gload(dreg, gTp + (size_t)J * 3 * TS); // D_J
            // L_J = F_{J-1} G_{J-1}
            t.rzero(acc);
            t.mma_tu(acc, sF, sG); // A(J, J-1) is upper triangular (KB >= kl)
            __syncthreads();
            t.rstore_t(sF, acc); // sF now holds L_J, transposed
            t.gstore_t(gL + tb + J * TS, acc);
            __syncthreads();
            // S_J = D_J - L_J E_{J-1}
#pragma unroll
            for (int i = 0; i < TL::TR; i++)
#pragma unroll
                for (int j = 0; j < TL::TC; j++) acc[i][j] = dreg[i][j];
            t.mms_t_bl(acc, sF, sE); // A(J-1, J) is lower triangular
            __syncthreads(); // sF, sE and sG are free from here on
            cp_async_tile<T, KB, NT>(sE, gTp + (size_t)J * 3 * TS + 2 * TS); // E_J
            if (J + 1 < N) cp_async_tile<T, KB, NT>(sF, gTp + (size_t)(J + 1) * 3 * TS + TS);
            cp_async_commit();
        }
        // G_J = S_J^{-1}
        ok = t.inverse(acc, buf) && ok;
        cp_async_wait_all();
        t.rstore(sG, acc);
        t.gstore_t(gG + tb + J * TS, acc); // column-major for the backward sweep
        __syncthreads();
    }
    if (!ok && threadIdx.x == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

// W forward sweep z_J = -L_J z_{J-1} (z_0 = C^, written by k_band_tiles) of
// partition blockIdx.x + 1 (partition 0 has no W spike); the next L tile
// streams into the second buffer while the current one is applied.
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_wsweep_big(const int *__restrict__ blk_off, const T *__restrict__ gL, T *gZ)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    const int part = blockIdx.x + 1;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;

    extern __shared__ char smraw[];
    T *sZ = (T *)smem_align(smraw), *sL0 = sZ + TL::ELEMS, *sL1 = sL0 + TL::ELEMS;
    TL t(threadIdx.x);
    typename TL::Reg acc;

    cp_async_tile<T, KB, NT>(sZ, gZ + tb);
    if (N > 1) cp_async_tile<T, KB, NT>(sL1, gL + tb + TS);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    for (int J = 1; J < N; J++) {
        T *cur = (J & 1) ? sL1 : sL0, *nxt = (J & 1) ? sL0 : sL1;
        if (J + 1 < N) cp_async_tile<T, KB, NT>(nxt, gL + tb + (size_t)(J + 1) * TS);
        cp_async_commit();
        t.rzero(acc);
        t.mms_t(acc, cur, sZ); // cur holds L_J transposed
        __syncthreads();
        t.rstore(sZ, acc);
        t.gstore(gZ + tb + J * TS, acc);
        cp_async_wait_all();
        __syncthreads();
    }
}

// Backward sweep X_J = G_J (Z_J - E_J X_{J+1}); blockIdx.y = 0: V of
// partition blockIdx.x, 1: its W.  Z_J comes from global memory into
// registers; G_{J-1} and E_{J-1} stream in as soon as G_J / E_J are used.
// gZ and gW are the same buffer (Z_J is read before X_J overwrites it).
template <class T, int KB>
__global__ void __launch_bounds__(NTOf<KB>::value)
    k_factor_bwd_big(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                     const T *__restrict__ gL, const T *__restrict__ gG, const T *__restrict__ gE, const T *gZ,
                     const T *__restrict__ gBhat, T *gV, T *gW)
{
    constexpr int NT = NTOf<KB>::value;
    using TL = Tile<T, KB, NT>;
    constexpr size_t TS = (size_t)KB * KB;
    constexpr int LD = TileLD<T, KB>::value;
    const bool isV = blockIdx.y == 0;
    const int part = blockIdx.x;
    if (isV ? part >= p - 1 : part == 0) return; // the whole CTA: no spike to compute
    const int s = part_start[part], e = part_start[part + 1], m = e - s;
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;

    extern __shared__ char smraw[];
    T *sG = (T *)smem_align(smraw), *sE = sG + TL::ELEMS, *sX = sE + TL::ELEMS;
    TL t(threadIdx.x);
    typename TL::Reg acc;

    // V's right-hand side [0; B^] is nonzero only in the last KB real rows:
    // blocks J0 and J0+1 (when m is not a multiple of KB).  Their forward-swept
    // values go to gV tiles J0 / J0+1 (row-major scratch, read back below).
    const int J0 = (m - KB) / KB, o = (m - KB) - J0 * KB;
    if (isV) {
        for (int q = threadIdx.x; q < KB * KB; q += NT) {
            const int r = q / KB, c = q - r * KB;
            // (o < 0: a partition shorter than a tile takes B^'s last m rows)
            sX[r * LD + c] = (r >= o && r - o < KB) ? gBhat[(size_t)part * TS + (r - o) * KB + c] : sc_zero<T>();
        }
        if (o > 0) {
            cp_async_tile<T, KB, NT>(sG, gL + tb + (J0 + 1) * TS); // L_{J0+1}, transposed
            cp_async_commit();
            for (int q = threadIdx.x; q < KB * KB; q += NT) {
                const int r = q / KB, c = q - r * KB;
                sE[r * LD + c] = r < o ? gBhat[(size_t)part * TS + (KB - o + r) * KB + c] : sc_zero<T>();
            }
            cp_async_wait_all();
        }
        __syncthreads();
        store_tile<T, KB>(gV + tb + J0 * TS, sX);
        if (o > 0) {
            // z_{J0+1} = [B^ rows KB-o..KB-1 ; 0] - L_{J0+1} z_{J0}
            t.rload(acc, sE);
            t.mms_t(acc, sG, sX);
            t.gstore(gV + tb + (J0 + 1) * TS, acc);
        }
        __syncthreads();
    }

    T *gX = isV ? gV : gW;
    cp_async_tile<T, KB, NT>(sG, gG + tb + (size_t)(N - 1) * TS);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    for (int J = N - 1; J >= 0; J--) {
        // T = Z_J - E_J X_{J+1}
        if (!isV)
            t.gload(acc, gZ + tb + J * TS);
        else if (J == J0 || (o > 0 && J == J0 + 1))
            t.gload(acc, gV + tb + J * TS);
        else
            t.rzero(acc);
        if (J < N - 1) t.mms_tl(acc, sE, sX); // A(J, J+1) is lower triangular (KB >= ku)
        __syncthreads();
        if (J > 0) {
            cp_async_tile<T, KB, NT>(sE, gE + tb + (size_t)(J - 1) * TS);
            cp_async_commit();
        }
        t.rstore(sX, acc);
        __syncthreads();
        // X_J = G_J T
        t.rzero(acc);
        t.mma_t(acc, sG, sX);
        __syncthreads();
        if (J > 0) {
            cp_async_tile<T, KB, NT>(sG, gG + tb + (size_t)(J - 1) * TS);
            cp_async_commit();
        }
        t.rstore(sX, acc);
        t.gstore_t(gX + tb + J * TS, acc); // column-major, for the tips and the retrieval
        cp_async_wait_all();
        __syncthreads();
    }
}

// ------------------------------------------------------------ small bands
// KB <= 4: a CTA per partition would leave most threads idle and pay a barrier
// per tile step.  KB lanes run one partition chain instead: lane r owns row r
// of every tile, the other rows arrive by shuffles (row_mul / row_msub /
// row_inv), and the chain's next DEPTH-1 blocks stream into its shared-memory
// ring by cp.async (each lane copies every KB-th 16-byte piece; __syncwarp on
// the segment publishes them).  Same recurrences and global layouts as
// k_factor_fwd / k_factor_bwd.
template <class T, int KB> struct QuadFwd {
    static constexpr int TS = KB * KB;
    static constexpr int DEPTH = 4;
    static constexpr int STAGE = 3 * TS;                             // D, F^T, E
    static constexpr int SLOT = DEPTH * STAGE * (int)sizeof(T) + 16; // per chain (odd in 16-byte units)
    static constexpr int CPC = chain_threads(SLOT);                  // chains per CTA
    static constexpr int NT = CPC * KB;
    static constexpr size_t SMEM = (size_t)CPC * SLOT;
};

template <class T, int KB>
__global__ void __launch_bounds__(QuadFwd<T, KB>::NT)
    k_quad_fwd(const T *__restrict__ gT, const int *__restrict__ blk_off, int p, T *gL, T *gG, T *gZ, unsigned *err)
{
    using C = QuadFwd<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH;
    constexpr int CH = C::STAGE * (int)sizeof(T) / 16;
    extern __shared__ __align__(16) char smc[];
    const int part = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int r = threadIdx.x % KB;
    if (part >= p) return; // whole segments leave together; no CTA barriers below
    const unsigned m = seg_mask<KB>();
    T *slot = (T *)(smc + (threadIdx.x / KB) * C::SLOT);
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    const T *gTp = gT + (size_t)blk_off[part] * C::STAGE;
    const bool doW = part > 0;
    auto issue = [&](int j) {
        if (j < N)
            for (int q = r; q < CH; q += KB)
                cp_async16((char *)(slot + (j % D) * C::STAGE) + 16 * q,
                           (const char *)(gTp + (size_t)j * C::STAGE) + 16 * q);
        cp_async_commit();
    };
    T g[KB], ep[KB], zp[KB];
#pragma unroll
    for (int c = 0; c < KB; c++) {
        g[c] = ep[c] = sc_zero<T>();
        zp[c] = doW ? gZ[tb + r * KB + c] : sc_zero<T>(); // z_0 = C^
    }
    bool ok = true;
#pragma unroll
    for (int j = 0; j < D - 1; j++) issue(j);
    for (int J = 0; J < N; J++) {
        issue(J + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
        const T *sc = slot + (J % D) * C::STAGE;
        T sr[KB];
#pragma unroll
        for (int c = 0; c < KB; c++) sr[c] = sc[r * KB + c]; // D_J
        if (J > 0) {
            T f[KB], l[KB];
#pragma unroll
            for (int c = 0; c < KB; c++) f[c] = sc[TS + c * KB + r]; // row r of F (stored as F^T)
            row_mul<T, KB>(m, l, f, g);                                // L_J = F_{J-1} G_{J-1}
#pragma unroll
            for (int c = 0; c < KB; c++) gL[tb + (size_t)J * TS + c * KB + r] = l[c];
            row_msub<T, KB>(m, sr, l, ep); // S_J = D_J - L_J E_{J-1}
            if (doW) {
                T z[KB];
#pragma unroll
                for (int c = 0; c < KB; c++) z[c] = sc_zero<T>();
                row_msub<T, KB>(m, z, l, zp); // z_J = -L_J z_{J-1}
#pragma unroll
                for (int c = 0; c < KB; c++) {
                    gZ[tb + (size_t)J * TS + r * KB + c] = z[c];
                    zp[c] = z[c];
                }
            }
        }
#pragma unroll
        for (int c = 0; c < KB; c++) ep[c] = sc[2 * TS + r * KB + c]; // E_J, for the next block
        __syncwarp(m); // the ring entry may be refilled from here on
        ok = row_inv<T, KB>(m, sr, r) && ok;
#pragma unroll
        for (int c = 0; c < KB; c++) {
            gG[tb + (size_t)J * TS + c * KB + r] = sr[c];
            g[c] = sr[c];
        }
    }
    cp_async_wait_all();
    if (!ok && r == 0) atomicOr(err, SPK_DEV_ERR_PIVOT);
}

template <class T, int KB> struct QuadBwd {
    static constexpr int TS = KB * KB;
    static constexpr int DEPTH = 4;
    static constexpr int STAGE = 3 * TS; // G, E, Z (W) / G, E (V)
    static constexpr int SLOT = DEPTH * STAGE * (int)sizeof(T) + 16;
    static constexpr int CPC = chain_threads(SLOT);
    static constexpr int NT = CPC * KB;
    static constexpr size_t SMEM = (size_t)CPC * SLOT;
};

// X_J = G_J (Z_J - E_J X_{J+1}), KB lanes per (partition, spike) chain, V and
// W of a partition on adjacent segments; blocks visited from N-1 down.
template <class T, int KB>
__global__ void __launch_bounds__(QuadBwd<T, KB>::NT)
    k_quad_bwd(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p, const T *__restrict__ gL,
               const T *__restrict__ gG, const T *__restrict__ gE, const T *__restrict__ gZ,
               const T *__restrict__ gBhat, T *gV, T *gW)
{
    using C = QuadBwd<T, KB>;
    constexpr int TS = C::TS, D = C::DEPTH;
    constexpr int CT = TS * (int)sizeof(T) / 16; // 16-byte pieces per tile
    extern __shared__ __align__(16) char smc[];
    const int ch = (blockIdx.x * blockDim.x + threadIdx.x) / KB;
    const int r = threadIdx.x % KB;
    const int part = ch >> 1;
    const bool isW = ch & 1;
    if (part >= p || (isW ? part == 0 : part == p - 1)) return; // whole segments; no CTA barriers below
    const unsigned m = seg_mask<KB>();
    T *slot = (T *)(smc + (threadIdx.x / KB) * C::SLOT);
    const int mrows = part_start[part + 1] - part_start[part];
    const int N = blk_off[part + 1] - blk_off[part];
    const size_t tb = (size_t)blk_off[part] * TS;
    T *gX = isW ? gW : gV;
    // step i handles block N-1-i; its tiles sit in ring entry i % D
    auto issue = [&](int i) {
        if (i < N) {
            const int J = N - 1 - i;
            char *st = (char *)(slot + (i % D) * C::STAGE);
            for (int q = r; q < CT; q += KB) {
                cp_async16(st + 16 * q, (const char *)(gG + tb + (size_t)J * TS) + 16 * q);
                cp_async16(st + TS * sizeof(T) + 16 * q, (const char *)(gE + tb + (size_t)J * TS) + 16 * q);
                if (isW)
                    cp_async16(st + 2 * TS * sizeof(T) + 16 * q, (const char *)(gZ + tb + (size_t)J * TS) + 16 * q);
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int i = 0; i < D - 1; i++) issue(i);
    // V's right-hand side [0; B^] lives in the last KB real rows: blocks J0
    // (rows o..KB-1) and J0+1 (rows 0..o-1, when o > 0).  A partition shorter
    // than a tile (o < 0) takes B^'s last m rows.
    T z0[KB], z1[KB];
    const int J0 = mrows >= KB ? (mrows - KB) / KB : 0;
    const int o = mrows - KB - J0 * KB;
#pragma unroll
    for (int c = 0; c < KB; c++) z0[c] = z1[c] = sc_zero<T>();
    if (!isW) {
        const T *B = gBhat + (size_t)part * TS;
#pragma unroll
        for (int c = 0; c < KB; c++) {
            z0[c] = (r >= o && r - o < KB) ? B[(r - o) * KB + c] : sc_zero<T>();
            z1[c] = r < o ? B[(KB - o + r) * KB + c] : sc_zero<T>();
        }
        if (o > 0) { // z_{J0+1} -= L_{J0+1} z_{J0}
            T l1[KB];
#pragma unroll
            for (int c = 0; c < KB; c++) l1[c] = gL[tb + (size_t)(J0 + 1) * TS + c * KB + r];
            row_msub<T, KB>(m, z1, l1, z0);
        }
    }
    T x[KB]; // row r of X_{J+1}
#pragma unroll
    for (int c = 0; c < KB; c++) x[c] = sc_zero<T>();
    for (int i = 0; i < N; i++) {
        const int J = N - 1 - i;
        issue(i + D - 1);
        cp_async_wait_n<D - 1>();
        __syncwarp(m);
        const T *sc = slot + (i % D) * C::STAGE;
        T t[KB], e[KB], g[KB];
#pragma unroll
        for (int c = 0; c < KB; c++) {
            t[c] = isW ? sc[2 * TS + r * KB + c] : (J == J0 ? z0[c] : (o > 0 && J == J0 + 1) ? z1[c] : sc_zero<T>());
            e[c] = sc[TS + c * KB + r]; // row r of E_J (stored column-major)
            g[c] = sc[c * KB + r];      // row r of G_J (stored column-major)
        }
        __syncwarp(m); // the ring entry may be refilled from here on
        if (J < N - 1) row_msub<T, KB>(m, t, e, x);
        row_mul<T, KB>(m, x, g, t);
#pragma unroll
        for (int c = 0; c < KB; c++) gX[tb + (size_t)J * TS + c * KB + r] = x[c];
    }
    cp_async_wait_all();
}

// Tips of V and W into the interface blocks of the reduced system (FP64):
//   P_i = V_i bottom, Q_i = W_{i+1} top, X_i = W_i bottom, Y_i = V_{i+1} top.
template <class T, int KB>
__global__ void k_tips(const int *__restrict__ part_start, const int *__restrict__ blk_off, int p,
                       const T *__restrict__ gV, const T *__restrict__ gW, typename HighOf<T>::type *RP,
                       typename HighOf<T>::type *RQ, typename HighOf<T>::type *RX,
                       typename HighOf<T>::type *RY)
{
    using H = typename HighOf<T>::type;
    constexpr size_t TS = (size_t)KB * KB;
    const int i = blockIdx.x; // interface i between partitions i and i+1
    const int mi = part_start[i + 1] - part_start[i];
    for (int q = threadIdx.x; q < KB * KB; q += blockDim.x) {
        const int r = q / KB, c = q - r * KB;
        // bottom rows of partition i: local row mi - KB + r
        // (a partition shorter than one tile -- only a batch's one-partition
        // system, whose spikes are zero -- has no distinct bottom tip)
        const int lb = mi - KB + r, Jb = lb / KB, rb = lb - Jb * KB;
        const bool hb = lb >= 0;
        const size_t ib = hb ? ((size_t)blk_off[i] + Jb) * TS + (size_t)c * KB + rb : 0;
        // top rows of partition i+1: local row r (block 0)
        const size_t it = (size_t)blk_off[i + 1] * TS + (size_t)c * KB + r;
        RP[(size_t)i * TS + q] = hb ? cvt_fast<H, T>(gV[ib]) : sc_zero<H>();
        RQ[(size_t)i * TS + q] = cvt_fast<H, T>(gW[it]);
        RX[(size_t)i * TS + q] = (i > 0 && hb) ? cvt_fast<H, T>(gW[ib]) : sc_zero<H>();
        RY[(size_t)i * TS + q] = (i + 1 < p - 1) ? cvt_fast<H, T>(gV[it]) : sc_zero<H>();
    }
}

template <class T, int KB> int run_tips(spk_plan *P, cudaStream_t st)
{
    using H = typename HighOf<T>::type;
    if (P->n_iface <= 0) return SPK_OK;
    k_tips<T, KB><<<P->n_iface, 256, 0, st>>>(P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_V,
                                              (const T *)P->d_W, (H *)P->d_RP, (H *)P->d_RQ, (H *)P->d_RX,
                                              (H *)P->d_RY);
    SPK_CHECK_LAUNCH();
    P->launches++;
    return SPK_OK;
}

// Partitions [part0, part1) of a two-sided plan: their band tiles (the rows'
// CSR entries must be on the device), both chains, the spikes' sweeps, the
// middle blocks and the back substitution.  The tips follow once every range
// is done.  The kernel attributes are set by a full run_factor first.
template <class T, int KB> int run_factor_range(spk_plan *P, const int *rowptr, const int *colind, const void *aij,
                                                int part0, int part1, cudaStream_t st)
{
    if (!P->twist || part0 < 0 || part1 > P->p || part0 >= part1) return SPK_EARG;
    const size_t TS = (size_t)KB * KB;
    const int b0 = P->blk_off[part0], b1 = P->blk_off[part1];
    if (cudaMemsetAsync((T *)P->d_Bhat + (size_t)part0 * TS, 0, sizeof(T) * TS * (part1 - part0), st) != cudaSuccess)
        return SPK_ECUDA;
    if (const int rc_ = launch_band_tiles<T, KB>(P, rowptr, colind, aij, b0, b1, st); rc_ != SPK_OK) return rc_;
    P->launches++;
    int rc = spk_twist_factor(P, 1, part0, part1, st);
    if (rc == SPK_OK) rc = spk_twist_factor(P, 0, part0, part1, st);
    return rc;
}

template <class T, int KB> int run_factor(spk_plan *P, const int *rowptr, const int *colind, const void *aij,
                                          cudaStream_t st)
{
    using H = typename HighOf<T>::type;
    constexpr int NT = NTOf<KB>::value;
    using S = FactorSmem<T, KB>;
    static bool attr = false;
    if (!attr) {
        if constexpr (S::BIG) {
            if (cudaFuncSetAttribute(k_factor_fwd_big<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)S::fwd) != cudaSuccess ||
                cudaFuncSetAttribute(k_wsweep_big<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)S::bwd) != cudaSuccess ||
                cudaFuncSetAttribute(k_factor_bwd_big<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)S::bwd) != cudaSuccess ||
                cudaFuncSetAttribute(k_band_tiles<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)S::band) != cudaSuccess)
                return SPK_ECUDA;
        } else {
        if constexpr (KB <= 4) {
            if (cudaFuncSetAttribute(k_quad_fwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)QuadFwd<T, KB>::SMEM) != cudaSuccess ||
                cudaFuncSetAttribute(k_quad_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)QuadBwd<T, KB>::SMEM) != cudaSuccess)
                return SPK_ECUDA;
        }
        if (cudaFuncSetAttribute(k_factor_fwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::fwd) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_band_tiles<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::band) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_factor_bwd<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bwd) !=
                cudaSuccess)
            return SPK_ECUDA;
        }
        attr = true;
    }
    const size_t TS = (size_t)KB * KB;
    if (cudaMemsetAsync(P->d_Bhat, 0, sizeof(T) * TS * P->p, st) != cudaSuccess) return SPK_ECUDA;
    spk_phase_begin(P, SPK_PH_BAND_TILES, st);
    if (const int rc_ = launch_band_tiles<T, KB>(P, rowptr, colind, aij, 0, P->total_blocks, st); rc_ != SPK_OK)
        return rc_;
    spk_phase_end(P, st);
    if (P->twist) { // two-sided chains (spike_twist.cu)
        P->launches++;  // k_band_tiles
        spk_phase_begin(P, SPK_PH_FACTOR_FWD, st);
        int rc = spk_twist_factor(P, 1, 0, P->p, st);
        spk_phase_end(P, st);
        if (rc != SPK_OK || P->p < 2) return rc;
        spk_phase_begin(P, SPK_PH_FACTOR_BWD, st);
        rc = spk_twist_factor(P, 0, 0, P->p, st);
        if (rc != SPK_OK) return rc;
        rc = run_tips<T, KB>(P, st);
        spk_phase_end(P, st);
        return rc;
    }
    spk_phase_begin(P, SPK_PH_FACTOR_FWD, st);
    if constexpr (S::BIG) {
        k_factor_fwd_big<T, KB><<<P->p, NT, S::fwd, st>>>((const T *)P->d_T, P->d_blk_off, (T *)P->d_L,
                                                          (T *)P->d_G, P->d_err);
        if (P->p > 1) {
            SPK_CHECK_LAUNCH();
            k_wsweep_big<T, KB><<<P->p - 1, NT, S::bwd, st>>>(P->d_blk_off, (const T *)P->d_L, (T *)P->d_W);
            P->launches++;
        }
    } else if constexpr (KB <= 4) {
        using CF = QuadFwd<T, KB>;
        const int cpc = chains_per_cta(P->p, CF::CPC);
        k_quad_fwd<T, KB><<<(P->p + cpc - 1) / cpc, cpc * KB, (size_t)cpc * CF::SLOT, st>>>(
            (const T *)P->d_T, P->d_blk_off, P->p, (T *)P->d_L, (T *)P->d_G, (T *)P->d_W, P->d_err);
    } else {
        k_factor_fwd<T, KB><<<P->p, NT, S::fwd, st>>>((const T *)P->d_T, P->d_blk_off, (T *)P->d_L, (T *)P->d_G,
                                                      (T *)P->d_W, P->d_err);
    }
    SPK_CHECK_LAUNCH();
    spk_phase_end(P, st);
    P->launches += 2;
    if (P->p > 1) {
        spk_phase_begin(P, SPK_PH_FACTOR_BWD, st);
        if constexpr (S::BIG) {
            k_factor_bwd_big<T, KB><<<dim3(P->p, 2), NT, S::bwd, st>>>(
                P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_L, (const T *)P->d_G, (const T *)P->d_E,
                (const T *)P->d_W, (const T *)P->d_Bhat, (T *)P->d_V, (T *)P->d_W);
        } else if constexpr (KB <= 4) {
            using CB = QuadBwd<T, KB>;
            const int cpc = chains_per_cta(2LL * P->p, CB::CPC);
            k_quad_bwd<T, KB><<<(2 * P->p + cpc - 1) / cpc, cpc * KB, (size_t)cpc * CB::SLOT, st>>>(
                P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_L, (const T *)P->d_G, (const T *)P->d_E,
                (const T *)P->d_W, (const T *)P->d_Bhat, (T *)P->d_V, (T *)P->d_W);
        } else {
            k_factor_bwd<T, KB><<<P->p, NT, S::bwd, st>>>(P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_L,
                                                          (const T *)P->d_G, (const T *)P->d_E, (T *)P->d_W,
                                                          (const T *)P->d_Bhat, (T *)P->d_V, (T *)P->d_W);
        }
        SPK_CHECK_LAUNCH();
        k_tips<T, KB><<<P->n_iface, 256, 0, st>>>(P->d_part_start, P->d_blk_off, P->p, (const T *)P->d_V,
                                                  (const T *)P->d_W, (H *)P->d_RP, (H *)P->d_RQ, (H *)P->d_RX,
                                                  (H *)P->d_RY);
        SPK_CHECK_LAUNCH();
        spk_phase_end(P, st);
        P->launches += 2;
    }
    return SPK_OK;
}

template <class T> int dispatch_factor(spk_plan *P, const int *rp, const int *ci, const void *a, cudaStream_t st)
{
    switch (P->KB) {
    case 2: return run_factor<T, 2>(P, rp, ci, a, st);
    case 4: return run_factor<T, 4>(P, rp, ci, a, st);
    case 8: return run_factor<T, 8>(P, rp, ci, a, st);
    case 16: return run_factor<T, 16>(P, rp, ci, a, st);
    case 32: return run_factor<T, 32>(P, rp, ci, a, st);
    case 64:
        if constexpr (sizeof(T) <= 8) return run_factor<T, 64>(P, rp, ci, a, st);
        else return SPK_EBAND;
    case 128:
        if constexpr (std::is_same<T, float>::value) return run_factor<T, 128>(P, rp, ci, a, st);
        else return SPK_EBAND;
    default: return SPK_EBAND;
    }
}

template <class T> int dispatch_range(spk_plan *P, const int *rp, const int *ci, const void *a, int p0, int p1,
                                     cudaStream_t st)
{
    switch (P->KB) {
    case 16: return run_factor_range<T, 16>(P, rp, ci, a, p0, p1, st);
    case 32: return run_factor_range<T, 32>(P, rp, ci, a, p0, p1, st);
    case 64:
        if constexpr (sizeof(T) <= 8) return run_factor_range<T, 64>(P, rp, ci, a, p0, p1, st);
        else return SPK_EBAND;
    default: return SPK_EARG;
    }
}

template <class T> int dispatch_tips(spk_plan *P, cudaStream_t st)
{
    switch (P->KB) {
    case 16: return run_tips<T, 16>(P, st);
    case 32: return run_tips<T, 32>(P, st);
    case 64:
        if constexpr (sizeof(T) <= 8) return run_tips<T, 64>(P, st);
        else return SPK_EBAND;
    default: return SPK_EARG;
    }
}

template <class T> size_t smem_for(int KB)
{
    switch (KB) {
    case 2: return FactorSmem<T, 2>::fwd;
    case 4: return FactorSmem<T, 4>::fwd;
    case 8: return FactorSmem<T, 8>::fwd;
    case 16: return FactorSmem<T, 16>::fwd;
    case 32: return FactorSmem<T, 32>::fwd;
    case 64:
        if constexpr (sizeof(T) <= 8) return FactorSmem<T, 64>::fwd;
        else return 0;
    case 128: // real mixed precision only (a 128-row FP64 or complex tile does not fit three times)
        if constexpr (std::is_same<T, float>::value) return FactorSmem<T, 128>::fwd;
        else return 0;
    default: return 0;
    }
}

} // namespace

extern "C" size_t spk_factor_smem(int KB, int is_complex, int mode)
{
    if (is_complex) return mode == SPK_MIXED ? smem_for<cfloat>(KB) : smem_for<cdouble>(KB);
    return mode == SPK_MIXED ? smem_for<float>(KB) : smem_for<double>(KB);
}

extern "C" int spk_factor_range(spk_plan *P, const int *d_rowptr, const int *d_colind, const void *d_aij, int part0,
                                int part1, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (P->is_complex)
        return P->mode == SPK_MIXED ? dispatch_range<cfloat>(P, d_rowptr, d_colind, d_aij, part0, part1, st)
                                    : dispatch_range<cdouble>(P, d_rowptr, d_colind, d_aij, part0, part1, st);
    return P->mode == SPK_MIXED ? dispatch_range<float>(P, d_rowptr, d_colind, d_aij, part0, part1, st)
                                : dispatch_range<double>(P, d_rowptr, d_colind, d_aij, part0, part1, st);
}

extern "C" int spk_factor_tips(spk_plan *P, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (P->is_complex) return P->mode == SPK_MIXED ? dispatch_tips<cfloat>(P, st) : dispatch_tips<cdouble>(P, st);
    return P->mode == SPK_MIXED ? dispatch_tips<float>(P, st) : dispatch_tips<double>(P, st);
}

extern "C" int spk_factor(spk_plan *P, const int *d_rowptr, const int *d_colind, const void *d_aij, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (P->is_complex)
        return P->mode == SPK_MIXED ? dispatch_factor<cfloat>(P, d_rowptr, d_colind, d_aij, st)
                                    : dispatch_factor<cdouble>(P, d_rowptr, d_colind, d_aij, st);
    return P->mode == SPK_MIXED ? dispatch_factor<float>(P, d_rowptr, d_colind, d_aij, st)
                                : dispatch_factor<double>(P, d_rowptr, d_colind, d_aij, st);
}
