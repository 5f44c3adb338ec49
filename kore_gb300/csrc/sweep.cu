// Solves with the block-cyclic-reduction factors of factor.cu, sparse products and
// the FP64 refinement loop.
//
// (A - sigma B) x = b with row scaling R and s = ||b||_inf (keeps complex64 in range):
// the right-hand side c = s^-1 R b is reduced level by level exactly as the blocks were,
//     level l, odd blocks j:   z_j = D_j^-1 f_j
//     level l, even blocks i:  f_i <- f_i - L_i z_jl - U_i z_jr        (CSR couplings at level 0)
// the last block is solved, x_0 = D_0^-1 f_0, and the levels are unwound in reverse,
//     level l >= 1, odd blocks j:   x_j = z_j - G_j x_jl - H_j x_jr,
//     level 0, odd blocks j:        g_j = c_j - L_j x_{j-1} - U_j x_{j+1},  x_j = D_j^-1 g_j
// then x <- s x.  At level 0 the couplings are sparse, so forming g_j from them and
// multiplying by D_j^-1 reads one dense block instead of the two of G_j, H_j.  One cooperative persistent kernel runs all phases (about 3 log2 K of
// them) as a dataflow over tiles of 32 rows: a tile starts as soon as the blocks it
// reads are complete (per-block completion counters), and the factor blocks stream
// from HBM through shared memory by TMA.
//
// Every kernel here works on all factorised shifts at once (shift s: its own factors,
// row scales and vectors at offset s * stride), so a batch of forcing frequencies is
// one sweep launch.
//
// In mixed precision the factors are complex64 and the result is refined in FP64:
//     r = b - (A - sigma B) x,  x += M32^-1 r   until ||r||_inf <= tol (||M||_inf ||x||_inf + ||b||_inf).
#include "kore_internal.cuh"
#include "kore_tma.cuh"
#include <cstddef>
#include <map>
#include <mutex>
#include <tuple>

namespace {

__device__ __forceinline__ double2 ldcg(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2 *p) { return __ldcg(p); }
__device__ __forceinline__ double2 ldg(const double2 *p) { return __ldg(p); }
__device__ __forceinline__ float2 ldg(const float2 *p) { return __ldg(p); }
__device__ __forceinline__ void stcg(double2 *p, double2 v) { __stcg(p, v); }
__device__ __forceinline__ void stcg(float2 *p, float2 v) { __stcg(p, v); }

struct SweepArgs {
    int K, S, nlev, nshift;
    const BcrLevel *levs;
    const void *Dinv, *G, *H, *LU;
    int64_t f_stride, lu_stride;     // per-shift strides of the factor blocks (elements)
    const int *ell_col;              // level-0 couplings as padded rows (kore_plan::d_ell_*)
    const void *ell_val;
    int ell_w;
    int64_t ell_stride;              // per-shift stride of ell_val (elements)
    const double2 *b;                // nshift x np right-hand sides (complex128, padded)
    const double *rscale;            // nshift x np
    const double *bnorm;             // nshift scalings
    void *f, *z, *x;                 // nshift x np reduction vectors (factor precision)
    double2 *out;                    // nshift x np
    int accumulate;
    int *cnt;                        // completion counters: nshift x stages x K, zeroed before the launch
    int *err;
    const int *skip;                 // shift s is skipped when skip[s * skip_stride] != 0
    int skip_stride;
    unsigned live_mask;              // shift s (< 32) takes part only when bit s is set
    int *count;                      // sweeps that ran
    int *count_total;
};

constexpr int kMaxLevels = 24;

// bit s of a live-shift mask (shifts past 31 always take part)
__host__ __device__ __forceinline__ bool mask_has(unsigned mask, int64_t s) {
    return s >= 32 || ((mask >> s) & 1u);
}

__device__ __forceinline__ void st_release_cta(long long *p, long long v) {
    asm volatile("st.release.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(p)), "l"(v) : "memory");
}
__device__ __forceinline__ long long ld_acquire_cta(const long long *p) {
    long long v;
    asm volatile("ld.acquire.cta.shared::cta.b64 %0, [%1];" : "=l"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}

// Thread 0 waits (bounded) until *c >= target; on timeout or an earlier error the
// error flag is set and the caller goes on (its result is then wrong, but the kernel
// ends).
__device__ __forceinline__ void wait_count(const int *c, int target, int *err) {
    unsigned spins = 0;
    while (ld_relaxed_i32(c) < target) {
        if (ld_relaxed_i32(err) != 0) return;
        if (++spins > KORE_SPIN_LIMIT) { atomicCAS(err, 0, KORE_DEVERR_FLAG); return; }
        __nanosleep(32);
    }
    __threadfence();   // acquire: the producer's data is read after the counter
}

// ----------------------------------------------------------------------------- the sweep kernel
// The tiles (32 rows of one block) of all stages are numbered in a topological order
//     A_0, B_0, A_1, B_1, ..., A_{L-1}, B_{L-1}, top, C_{L-1}, ..., C_1, E_0, C_0
// (A: z_j = D_j^-1 f_j, B: f_i -= L_i z_jl + U_i z_jr, C: x_j = z_j - G_j x_jl - H_j x_jr
// at levels >= 1; E_0: g_j = c_j - L_j x_jl - U_j x_jr and C_0: x_j = D_j^-1 g_j)
// and CTA c takes tiles c, c + G, c + 2G, ...  A tile reads only blocks whose counters
// are complete (e.g. a B tile needs A of its two neighbours), and after its rows are
// written 1 is added to the counter of (stage, block).  Tiles are taken in increasing
// order by co-resident CTAs, so every wait is on a tile of a lower number that some
// CTA is processing or has processed: no deadlock, and adjacent stages overlap.
//
// A tile of A, C, top or B at levels >= 1 reads one or two S x S blocks (stored
// column-major); they are cut into chunks of 32 rows x kCols columns (16 KB) that one
// producer thread copies with cp.async.bulk.tensor into a ring of shared-memory slots,
// each slot guarded by a "full" mbarrier (completed by the copy) and an "empty"
// mbarrier (one arrival per consumer warp).  The producer runs ahead through the CTA's
// tile sequence: the factor data of later tiles does not depend on the sweep, so it is
// fetched while the consumer warps wait for their input vectors.  A dependency-checker
// warp also runs ahead and publishes in shared memory which tiles have their inputs
// complete.  B_0 and E_0 read the level-0 couplings as padded rows (at most a few
// dozen entries per row) with plain coalesced loads instead.
constexpr int kTmaConsumerWarps = 4;
constexpr int kTmaConsumers = 32 * kTmaConsumerWarps;
// Variants: 2, 3 or 4 CTAs per SM (deeper rings per CTA, or more CTAs whose per-tile
// work -- input vectors, reduction, signalling -- overlaps the others' streaming) and
// chunks of 8 or 16 KB (the ring holds the same bytes; with smaller chunks a consumed
// chunk frees its slot sooner, so more of the ring is in flight).  The autotuner below
// picks one per plan shape; untuned sweeps use 4 CTAs per SM and 8 KB chunks.
struct TmaVariant { int cps, chunk; };
constexpr TmaVariant kTmaVariants[] = {{2, 16384}, {3, 16384}, {4, 16384}, {2, 8192}, {3, 8192}, {4, 8192}};
constexpr TmaVariant kTmaDefault = {4, 8192};
constexpr int kTmaThreads = kTmaConsumers + 64;   // + one producer warp + one dependency-checker warp
constexpr int kTileRows = 32;
constexpr int kMaxRing = 24;
constexpr int kEllReg = 4;   // level-0 coupling entries per thread held in registers (width 32)
// input-vector loads in flight per consumer lane: a two-matrix tile's slice (about 2 S / 4
// entries per warp: 2 x 7 x 16 at S = 400 with 16 KB chunks, 2 x 13 x 8 with 8 KB) takes
// one round of L2 latency with 8, two with 4; the variants whose register budget
// (65536 / (192 CPS)) cannot hold 8 keep 4
template <typename C, int CPS> constexpr int fill_of() { return (CPS == 2 || (CPS == 3 && sizeof(C) == 8)) ? 8 : 4; }

enum { kMapDinv = 0, kMapG = 1, kMapH = 2, kMapLU = 3 };

struct SweepTmaParams {
    CUtensorMap maps[4];   // Dinv, G, H, LU: (2S reals, S columns, blocks, shifts)
    SweepArgs a;
    int nst;               // ring slots
};

template <typename C, int CHUNK> struct TmaShape {
    static constexpr int kCols = CHUNK / (kTileRows * (int)sizeof(C));   // columns per chunk
    static constexpr int kColsPerWarp = kCols / kTmaConsumerWarps;
};

// One tile of the sweep: stage kind (0 A, 1 B, 2 top, 3 C, 4 E_0), level, shift, block
// of its rows, first row, and the blocks it multiplies (map, block index within the map).
struct TileJob {
    int kind, l, nmat, r0;
    int64_t s, blk;
    int map[2];
    int64_t mblk[2];
    int64_t vblk[2];     // block of the vector each matrix multiplies
    bool hasl, hasr;
};

__device__ __forceinline__ void decode_tile(int64_t g, int &k, const int64_t *st_begin, const BcrLevel *lv_s, int L,
                                            int ntile, TileJob &t) {
    while (g >= st_begin[k + 1]) ++k;
    const int64_t loc = g - st_begin[k];
    if (k < 2 * L) { t.kind = (k & 1) ? 1 : 0; t.l = k >> 1; }
    else if (k == 2 * L) { t.kind = 2; t.l = L; }
    else if (k < 3 * L) { t.kind = 3; t.l = 3 * L - k; }
    else if (k == 3 * L) { t.kind = 4; t.l = 0; }
    else { t.kind = 3; t.l = 0; }
    const int nblk = (t.kind == 1) ? lv_s[t.l].neven : (t.kind == 2 ? 1 : lv_s[t.l].nodd);
    t.s = loc / ((int64_t)nblk * ntile);
    const int64_t rem = loc - t.s * nblk * ntile;
    const int64_t bi = rem / ntile;
    t.r0 = (int)(rem - bi * ntile) * kTileRows;
    t.nmat = 0;
    t.hasl = t.hasr = false;
    if (t.kind == 0) {
        const int64_t j = (2 * bi + 1) * lv_s[t.l].stride;
        t.blk = j;
        t.map[0] = kMapDinv; t.mblk[0] = j; t.vblk[0] = j; t.nmat = 1;
    } else if (t.kind == 1) {
        const BcrLevel lv = lv_s[t.l];
        const int64_t q = 2 * bi;
        t.blk = q * lv.stride;
        t.hasl = q >= 1;
        t.hasr = q + 1 < lv.Kl;
        if (t.l > 0) {
            // L_q z_jl first when it exists, then U_q z_jr
            const int64_t jl = (q - 1) * lv.stride, jr = (q + 1) * lv.stride;
            t.map[0] = t.map[1] = kMapLU;
            t.mblk[0] = t.hasl ? lv.lu_L + q : lv.lu_U + q;
            t.vblk[0] = t.hasl ? jl : jr;
            t.mblk[1] = lv.lu_U + q;
            t.vblk[1] = jr;
            t.nmat = (int)t.hasl + (int)t.hasr;
        }
    } else if (t.kind == 2) {
        t.blk = 0;
        t.map[0] = kMapDinv; t.mblk[0] = 0; t.vblk[0] = 0; t.nmat = 1;
    } else if (t.kind == 3 && t.l > 0) {
        const BcrLevel lv = lv_s[t.l];
        const int64_t q = 2 * bi + 1, j = q * lv.stride;
        t.blk = j;
        t.hasr = q + 1 < lv.Kl;
        t.map[0] = kMapG; t.mblk[0] = j; t.vblk[0] = j - lv.stride; t.nmat = 1;
        if (t.hasr) { t.map[1] = kMapH; t.mblk[1] = j; t.vblk[1] = j + lv.stride; t.nmat = 2; }
    } else if (t.kind == 3) {
        // C_0: x_j = D_j^-1 g_j, g_j from E_0 in f
        const int64_t j = 2 * bi + 1;
        t.blk = j;
        t.map[0] = kMapDinv; t.mblk[0] = j; t.vblk[0] = j; t.nmat = 1;
    } else {
        // E_0: g_j = c_j - L_j x_{j-1} - U_j x_{j+1} from the padded coupling rows
        const int64_t q = 2 * bi + 1;
        t.blk = q;
        t.hasl = true;
        t.hasr = q + 1 < lv_s[0].Kl;
        t.vblk[0] = q - 1; t.vblk[1] = q + 1;
    }
}

template <typename C, int CPS, int CHUNK>
__global__ void __launch_bounds__(kTmaThreads, CPS) k_sweep_tma(const __grid_constant__ SweepTmaParams P) {
    using Shape = TmaShape<C, CHUNK>;
    constexpr int kCols = Shape::kCols, kCpw = Shape::kColsPerWarp;
    constexpr int kFill = fill_of<C, CPS>();
    const SweepArgs &a = P.a;
    const int nst = P.nst;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const int S = a.S, ns = a.nshift, L = a.nlev, K = a.K;
    const int nc = (S + kCols - 1) / kCols;   // chunks per block
    const int nvec = nc * kCols;
    unsigned char *ring = smem_raw;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + (size_t)nst * CHUNK);
    uint64_t *empty = full + nst;
    C *vbuf = reinterpret_cast<C *>(empty + nst);   // 2 x nvec input vectors (each warp fills its columns)
    __shared__ C red[2][kTmaConsumerWarps][33];   // per-warp partial sums, by tile parity
    __shared__ BcrLevel lv_s[kMaxLevels];
    __shared__ int64_t st_begin[3 * kMaxLevels + 2];
    __shared__ long long ready;      // highest tile of this CTA whose inputs are complete
    {
        bool all = true;
        for (int s = 0; s < ns; ++s)
            all = all && (!mask_has(a.live_mask, s) || (a.skip && a.skip[s * a.skip_stride] != 0));
        if (all) return;
    }
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (a.count && blockIdx.x == 0 && tid == 0) { atomicAdd(a.count, 1); atomicAdd(a.count_total, 1); }
    const int64_t np = (int64_t)K * S;
    const int ntile = (S + kTileRows - 1) / kTileRows;
    const int nstage = L > 0 ? 3 * L + 2 : 1;
    if (tid < L) lv_s[tid] = a.levs[tid];
    if (tid == 0) {
        for (int i = 0; i < nst; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], kTmaConsumerWarps); }
        mbar_fence_init();
        ready = -1;
    }
    if (tid == kTmaConsumers) for (int i = 0; i < 4; ++i) tma_prefetch_desc(&P.maps[i]);
    __syncthreads();
    if (tid == 0) {
        int64_t acc = 0;
        for (int k = 0; k < nstage; ++k) {
            st_begin[k] = acc;
            int nblk;
            if (k < 2 * L) nblk = (k & 1) ? lv_s[k >> 1].neven : lv_s[k >> 1].nodd;
            else if (k == 2 * L) nblk = 1;
            else if (k < 3 * L) nblk = lv_s[3 * L - k].nodd;
            else nblk = lv_s[0].nodd;   // E_0, C_0
            acc += (int64_t)nblk * ntile * ns;
        }
        st_begin[nstage] = acc;
    }
    __syncthreads();
    const int64_t total = st_begin[nstage];
    auto live = [&](int64_t s) -> bool {
        return mask_has(a.live_mask, s) && !(a.skip && a.skip[s * a.skip_stride] != 0);
    };
    auto ctr = [&](int64_t s, int sid, int64_t blk) -> int * { return a.cnt + ((s * nstage + sid) * K + blk); };
    auto xready = [&](int64_t s, int64_t blk) -> int * {
        if (blk == 0) return ctr(s, 2 * L, 0);
        const int lb = __ffsll(blk) - 1;
        return ctr(s, 2 * L + 1 + lb, blk);
    };

    if (w == kTmaConsumerWarps) {
        // ------------------------------------------------------------------ producer
        if (lane == 0) {
            uint32_t slot = 0, ph = 0;
            int k = 0;
            uint64_t issued = 0;
            TileJob t;
            for (int64_t g = blockIdx.x; g < total; g += gridDim.x) {
                decode_tile(g, k, st_begin, lv_s, L, ntile, t);
                if (!live(t.s)) continue;
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    if (m >= t.nmat) break;
                    for (int ch = 0; ch < nc; ++ch) {
                        if (!mbar_wait(&empty[slot], ph ^ 1)) atomicCAS(a.err, 0, KORE_DEVERR_FLAG);
                        mbar_arrive_expect_tx(&full[slot], CHUNK);
                        tma_load_4d(ring + (size_t)slot * CHUNK, &P.maps[t.map[m]], &full[slot],
                                    2 * t.r0, ch * kCols, (int)t.mblk[m], (int)t.s);
                        ++issued;
                        if (++slot == (uint32_t)nst) { slot = 0; ph ^= 1; }
                    }
                }
            }
            // every copy has landed before the CTA may exit (normally already consumed)
            const uint64_t first = issued > (uint64_t)nst ? issued - nst : 0;
            for (uint64_t i = first; i < issued; ++i)
                if (!mbar_wait(&full[i % nst], (uint32_t)((i / nst) & 1))) atomicCAS(a.err, 0, KORE_DEVERR_FLAG);
        }
        return;
    }
    auto vec = [&](void *base, int64_t s) -> C * { return static_cast<C *>(base) + s * np; };
    auto rhs0 = [&](int64_t s, int64_t p) -> C {
        const double bn = a.bnorm[s];
        const double bscale = (bn > 0.0) ? 1.0 / bn : 1.0;
        return from_c128<C>((a.rscale[s * np + p] * bscale) * a.b[s * np + p]);
    };

    if (w == kTmaConsumerWarps + 1) {
        // ------------------------------------------------------------------ dependency checker
        // Runs ahead of the consumers through the CTA's tiles: waits (bounded, one lane
        // per counter) for the completion counters of the blocks a tile reads and
        // publishes the tile in `ready`, so that the consumers find their inputs complete
        // without a round trip to global memory of their own.  A timed-out wait sets the
        // error flag and the tile is published all the same.
        int k = 0;
        TileJob t;
        for (int64_t g = blockIdx.x; g < total; g += gridDim.x) {
            decode_tile(g, k, st_begin, lv_s, L, ntile, t);
            const int64_t s = t.s;
            if (live(s)) {
                // the counters this tile needs (at most three), one lane waiting on each
                const int *d0 = nullptr, *d1 = nullptr, *d2 = nullptr;
                if (t.kind == 0) {
                    if (t.l > 0) d0 = ctr(s, L + t.l - 1, t.blk);
                } else if (t.kind == 1) {
                    const int64_t st = lv_s[t.l].stride;
                    if (t.hasl) d0 = ctr(s, t.l, t.blk - st);
                    if (t.hasr) d1 = ctr(s, t.l, t.blk + st);
                    if (t.l > 0) d2 = ctr(s, L + t.l - 1, t.blk);
                } else if (t.kind == 2) {
                    if (L > 0) d0 = ctr(s, 2 * L - 1, 0);
                } else if (t.kind == 4) {
                    d0 = xready(s, t.vblk[0]);
                    if (t.hasr) d1 = xready(s, t.vblk[1]);
                } else if (t.l == 0) {
                    d0 = ctr(s, 3 * L + 1, t.blk);
                } else {
                    d0 = xready(s, t.vblk[0]);
                    if (t.nmat > 1) d1 = xready(s, t.vblk[1]);
                }
                const int *mine = lane == 0 ? d0 : (lane == 1 ? d1 : (lane == 2 ? d2 : nullptr));
                if (mine) wait_count(mine, ntile, a.err);
                __syncwarp();
            }
            if (lane == 0) st_release_cta(&ready, (long long)g);
        }
        return;
    }

    // ---------------------------------------------------------------------- consumers
    // Each warp follows the CTA's tiles on its own: it waits for `ready`, loads the
    // entries of the input vectors that its columns of the chunks multiply, consumes
    // its columns of every chunk of the ring, and leaves its partial sums in red; one
    // named barrier per tile gathers them, after which warp 0 reduces and writes the
    // rows and signals the tile's completion while the other warps go on.
    auto emit = [&](int64_t s, int64_t p, C val, double2 prev) {
        stcg(vec(a.x, s) + p, val);
        const double bn = a.bnorm[s];
        const double2 d = ((bn > 0.0) ? bn : 1.0) * to_c128(val);
        a.out[s * np + p] = a.accumulate ? prev + d : d;
    };
    uint32_t slot = 0, ph = 0;
    int k = 0;
    TileJob t;
    int64_t i = 0;
    for (int64_t g = blockIdx.x; g < total; g += gridDim.x, ++i) {
        decode_tile(g, k, st_begin, lv_s, L, ntile, t);
        const int64_t s = t.s;
        const int sid = t.kind == 0 ? t.l
                      : (t.kind == 1 ? L + t.l : (t.kind == 2 ? 2 * L : (t.kind == 3 ? 2 * L + 1 + t.l : 3 * L + 1)));
        int *done = ctr(s, sid, t.blk);
        C (*rd)[33] = red[i & 1];
        if (live(s)) {
            // level-0 couplings (B_0, E_0): this thread's padded entries are loaded before
            // the wait, as they do not depend on the sweep; lane = row, warp w = entries w + 8u
            const bool ell = (t.kind == 1 && t.l == 0) || t.kind == 4;
            const int64_t ebase = (t.blk * ntile + t.r0 / kTileRows) * (int64_t)a.ell_w * 32 + lane;
            const C *ellv = static_cast<const C *>(a.ell_val) + s * a.ell_stride;
            int ecol[kEllReg];
            C eval[kEllReg];
#pragma unroll
            for (int u = 0; u < kEllReg; ++u) {
                const int kk = w + u * kTmaConsumerWarps;
                const bool in = ell && kk < a.ell_w;
                ecol[u] = in ? __ldg(a.ell_col + ebase + (int64_t)kk * 32) : -1;
                eval[u] = in ? ldg(ellv + ebase + (int64_t)kk * 32) : czero<C>();
            }
            if (lane == 0) {
                // the checker has seen this tile's inputs complete (acquire; __syncwarp
                // orders the rest of the warp after this lane)
                unsigned spins = 0;
                while (ld_acquire_cta(&ready) < (long long)g) {
                    if (++spins > KORE_SPIN_LIMIT) { atomicCAS(a.err, 0, KORE_DEVERR_FLAG); break; }
                    __nanosleep(16);
                }
            }
            __syncwarp();
            // rows this tile writes, and what the write combines with (read early)
            const int r = t.r0 + lane;
            const int64_t p = t.blk * S + r;
            const bool wr = w == 0 && r < S;
            C zf = czero<C>();
            double2 prev = mk(0.0, 0.0);
            if (wr) {
                if (t.kind == 1 && t.l > 0) zf = ldcg(vec(a.f, s) + p);
                else if (t.kind == 3 && t.l > 0) zf = ldcg(vec(a.z, s) + p);
                if ((t.kind == 2 || t.kind == 3) && a.accumulate) prev = a.out[s * np + p];
            }
            if (!ell && t.nmat > 0) {
                // this warp's slice of the input vectors: columns ch kCols + w kCpw + u
                const C *src = (t.kind == 0 || t.kind == 2 || (t.kind == 3 && t.l == 0))
                                   ? vec(a.f, s) : (t.kind == 1 ? vec(a.z, s) : vec(a.x, s));
                const bool from_b = (t.kind == 0 && t.l == 0) || (t.kind == 2 && L == 0);
                const double bn = a.bnorm[s];
                const double bscale = (bn > 0.0) ? 1.0 / bn : 1.0;
                const int per = nc * kCpw, ne = t.nmat * per;
                const int64_t vb0 = t.vblk[0] * S, vb1 = t.vblk[1] * S;
                for (int e0 = 0; e0 < ne; e0 += 32 * kFill) {
                    C v[kFill];
                    int cv[kFill];
#pragma unroll
                    for (int u = 0; u < kFill; ++u) {
                        const int e = e0 + u * 32 + lane;
                        const int m = e >= per ? 1 : 0, rem = e - m * per;
                        const int c = (rem / kCpw) * kCols + w * kCpw + rem % kCpw;
                        cv[u] = (e < ne) ? m * nvec + c : -1;
                        v[u] = czero<C>();
                        if (e < ne && c < S) {
                            const int64_t q = (m ? vb1 : vb0) + c;
                            v[u] = from_b ? from_c128<C>((a.rscale[s * np + q] * bscale) * a.b[s * np + q])
                                          : ldcg(src + q);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < kFill; ++u)
                        if (cv[u] >= 0) vbuf[cv[u]] = v[u];
                }
                __syncwarp();
            }
            C acc = czero<C>();
            if (ell) {
                const C *z = vec(t.kind == 4 ? a.x : a.z, s);   // E_0 couples to x, B_0 to z
#pragma unroll
                for (int u = 0; u < kEllReg; ++u)
                    if (ecol[u] >= 0) acc = cfma(acc, eval[u], ldcg(z + ecol[u]));
                for (int kk = w + kEllReg * kTmaConsumerWarps; kk < a.ell_w; kk += kTmaConsumerWarps) {
                    const int c = __ldg(a.ell_col + ebase + (int64_t)kk * 32);
                    if (c >= 0) acc = cfma(acc, ldg(ellv + ebase + (int64_t)kk * 32), ldcg(z + c));
                }
            } else if (t.nmat > 0) {
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    if (m >= t.nmat) break;
                    const C *vv = vbuf + m * nvec + w * kCpw;
                    for (int ch = 0; ch < nc; ++ch) {
                        if (!mbar_wait(&full[slot], ph)) atomicCAS(a.err, 0, KORE_DEVERR_FLAG);
                        const C *bc = reinterpret_cast<const C *>(ring + (size_t)slot * CHUNK) +
                                      w * kCpw * kTileRows + lane;
                        const C *vc = vv + ch * kCols;
#pragma unroll
                        for (int u = 0; u < kCpw; ++u) acc = cfma(acc, bc[u * kTileRows], vc[u]);
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&empty[slot]);
                        if (++slot == (uint32_t)nst) { slot = 0; ph ^= 1; }
                    }
                }
            }
            rd[w][lane] = acc;
            named_sync(1, kTmaConsumers);
            if (w == 0) {
                C val = czero<C>();
#pragma unroll
                for (int q = 0; q < kTmaConsumerWarps; ++q) val = val + rd[q][lane];
                if (wr) {
                    if (ell) stcg(vec(a.f, s) + p, rhs0(s, p) - val);
                    else if (t.kind == 0) stcg(vec(a.z, s) + p, val);
                    else if (t.kind == 1) stcg(vec(a.f, s) + p, zf - val);
                    else if (t.kind == 2 || t.l == 0) emit(s, p, val, prev);
                    else emit(s, p, zf - val, prev);
                }
            }
        }
        if (w == 0) {
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                atomicAdd(done, 1);
            }
        }
    }
}

// max |v_p| per shift: grid (x, shift) -> red[s * gridDim.x + blockIdx.x]
__global__ void k_absmax(int64_t np, const double2 *__restrict__ v, double *__restrict__ red) {
    const int64_t s = blockIdx.y;
    v += s * np;
    double mx = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x)
        mx = fmax(mx, fmax(fabs(v[p].x), fabs(v[p].y)));
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) red[s * gridDim.x + blockIdx.x] = t;
    }
}

// out[s] = max of in[s * n .. s * n + n), one CTA per shift
__global__ void k_reduce_max(const double *__restrict__ in, int n, double *__restrict__ out) {
    const int s = blockIdx.x;
    in += (int64_t)s * n;
    double mx = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, in[i]);
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) out[s] = t;
    }
}

// Sparse products y = B x, A x - lam B x and the refinement residual b - (A x - lam B x).
// On this GPU the FP64 pipe, not HBM, bounds them (about two FP64 multiply-adds per
// SM per clock), so A is stored as a real matrix split into real and imaginary
// coefficients (two multiply-adds per value instead of four for a complex entry),
// each row's real and imaginary segments summed separately and combined at the end.
// Rows are short (a few dozen values): one thread per row with kRowUnroll gathers in
// flight.  Splitting a row over 2 or 4 lanes costs FP64 additions to combine the
// partial sums, which take FP64-pipe issue slots like the products do (measured on
// the 240k-unknown shell: 4 lanes 179 ms, 2 lanes 140 ms, 1 lane 129 ms per solve).
// The tau-method boundary rows are dense over a radial expansion (hundreds of
// entries); rows with more than kKoreLongRow values (A + B) are listed at plan
// creation and done by a whole warp each in extra CTAs at the end of the grid, so that
// they do not hold back the CTAs of the short rows.
constexpr int kRowLanes = 1;   // threads per short row
constexpr int kRowUnroll = 4;

struct SpmvArgs {
    int64_t np;
    int S, K;               // padded block size, blocks: row p's columns lie in blocks p/S - 1 .. p/S + 1
    int mode;               // 0: y = B x.  1: y = A x - lam B x.  2: y = b - (A x - lam B x)
    int has_b;
    const int *srow, *smid, *scol;  // A split into real and imaginary coefficients (kore_plan::d_s*)
    const double *sval;
    const int *brow, *bcol;
    const double *bval;
    const int *long_rows;   // rows done by a warp each
    int nlong;
    int short_blocks;       // CTAs of the 4-lane part (the long-row CTAs follow)
    double2 lam;            // shift when sig is null
    const double2 *sig;     // per-shift shifts (shift = blockIdx.y)
    const double2 *x, *rhs;
    double2 *y;
    double *part;           // mode 2: per-CTA maxima of |y| and |x|, part[s * 2 gridDim.x + 2 blockIdx.x (+1)]
    const int *skip;        // shift s is skipped when skip[s * skip_stride] != 0
    int skip_stride;
    unsigned live_mask;     // shift s (< 32) is computed only when bit s is set
};

// The entries of x one CTA of short rows reads, staged in shared memory: columns
// [w0, w1) (block-aligned: the blocks of the CTA's rows and one on either side).  An
// entry outside the window (none for a plan, whose band check keeps every column in the
// neighbouring blocks) is read from global memory.
struct XWin {
    const double2 *__restrict__ sh;
    int64_t w0, w1;
    __device__ __forceinline__ double2 get(const double2 *__restrict__ x, int c) const {
        return (c >= w0 && c < w1) ? sh[c - w0] : __ldg(x + c);
    }
};

// acc += sum over the values sub, sub + LANES, ... of [e0, e1) of val[e] x[col[e]]
// (kRowUnroll loads in flight per lane, two FP64 multiply-adds per value); x entries from
// the window when one is given
template <int LANES, bool WIN>
__device__ __forceinline__ void seg_dot(const int *__restrict__ col, const double *__restrict__ val, int e0, int e1,
                                        int sub, const double2 *__restrict__ x, const XWin &xw, double2 &acc) {
    for (int e = e0 + sub; e < e1; e += LANES * kRowUnroll) {
        int c[kRowUnroll];
        double v[kRowUnroll];
#pragma unroll
        for (int u = 0; u < kRowUnroll; ++u) {
            const int q = e + u * LANES;
            c[u] = q < e1 ? __ldg(col + q) : -1;
            v[u] = q < e1 ? __ldg(val + q) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kRowUnroll; ++u)
            if (c[u] >= 0) {
                const double2 xv = WIN ? xw.get(x, c[u]) : __ldg(x + c[u]);
                acc.x = fma(v[u], xv.x, acc.x);
                acc.y = fma(v[u], xv.y, acc.y);
            }
    }
}

// Partial sums of row p: the real-coefficient values of A (sr), its imaginary-coefficient
// values (si: A x = sr + i si) and B (sb).
template <int LANES, bool WIN>
__device__ __forceinline__ void row_dot(const SpmvArgs &a, int64_t p, int sub, const double2 *__restrict__ x,
                                        const XWin &xw, double2 &sr, double2 &si, double2 &sb) {
    if (a.mode != 0) {
        const int em = a.smid[p];
        seg_dot<LANES, WIN>(a.scol, a.sval, a.srow[p], em, sub, x, xw, sr);
        seg_dot<LANES, WIN>(a.scol, a.sval, em, a.srow[p + 1], sub, x, xw, si);
    }
    if (a.has_b) seg_dot<LANES, WIN>(a.bcol, a.bval, a.brow[p], a.brow[p + 1], sub, x, xw, sb);
}

// x entries of the window of a CTA of 256 short rows: at most (255 / S + 4) blocks
__host__ __device__ __forceinline__ int64_t spmv_window(int S) { return (int64_t)(255 / S + 4) * S; }

// |v| of a double as the bits of its absolute value: for non-negative IEEE doubles the
// integer order is the numeric order, so maxima run on the integer units, not on the
// FP64 pipe, and a NaN (above +inf as bits) is kept instead of dropped as fmax drops it
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(256) k_spmv(SpmvArgs a) {
    extern __shared__ double2 xsh[];   // spmv_window(S) entries
    const int64_t s = blockIdx.y;
    if (!mask_has(a.live_mask, s) || (a.skip && a.skip[s * a.skip_stride])) return;
    const int64_t np = a.np;
    const double2 *x = a.x + s * np;
    double2 *y = a.y + s * np;
    const double2 *rhs = a.rhs ? a.rhs + s * np : nullptr;
    const double2 lam = a.sig ? a.sig[s] : a.lam;
    unsigned long long rmax = 0, xmax = 0;
    auto finish = [&](int64_t p, double2 sr, double2 si, double2 sb) {
        const double2 sa = mk(sr.x - si.y, sr.y + si.x);   // A x = sr + i si
        double2 v = (a.mode == 0) ? sb : sa - lam * sb;
        if (a.mode == 2) {
            v = rhs[p] - v;
            const double2 xp = x[p];
            rmax = max(rmax, max(abs_bits(v.x), abs_bits(v.y)));
            xmax = max(xmax, max(abs_bits(xp.x), abs_bits(xp.y)));
        }
        y[p] = v;
    };
    if ((int)blockIdx.x < a.short_blocks) {
        static_assert(kRowLanes == 1, "one thread per short row");
        // stage the x entries of the blocks this CTA's rows couple to (coalesced), so the
        // rows' gathers hit shared memory instead of waiting on L2
        const int64_t r0 = blockIdx.x * (int64_t)blockDim.x;
        const int64_t rl = ((r0 + blockDim.x < np) ? r0 + blockDim.x : np) - 1;
        const int64_t b0 = (r0 / a.S > 0) ? r0 / a.S - 1 : 0;
        const int64_t b1 = (rl / a.S + 1 < a.K) ? rl / a.S + 1 : a.K - 1;
        XWin xw{xsh, b0 * a.S, (b1 + 1) * a.S};
        for (int64_t c = xw.w0 + threadIdx.x; c < xw.w1; c += blockDim.x) xsh[c - xw.w0] = __ldg(x + c);
        __syncthreads();
        const int64_t p = r0 + threadIdx.x;
        bool live = p < np;
        if (live) {
            const int len = (a.srow[p + 1] - a.srow[p]) + (a.has_b ? a.brow[p + 1] - a.brow[p] : 0);
            live = len <= kKoreLongRow;
        }
        if (live) {
            double2 sr = mk(0.0, 0.0), si = mk(0.0, 0.0), sb = mk(0.0, 0.0);
            row_dot<1, true>(a, p, 0, x, xw, sr, si, sb);
            finish(p, sr, si, sb);
        }
    } else {
        const int lane = threadIdx.x & 31;
        const int wid = (blockIdx.x - a.short_blocks) * (blockDim.x >> 5) + (threadIdx.x >> 5);
        if (wid < a.nlong) {
            const int64_t p = a.long_rows[wid];
            double2 sr = mk(0.0, 0.0), si = mk(0.0, 0.0), sb = mk(0.0, 0.0);
            row_dot<32, false>(a, p, lane, x, XWin{nullptr, 0, 0}, sr, si, sb);
            sr = warp_sum(sr);
            si = warp_sum(si);
            sb = warp_sum(sb);
            if (lane == 0) finish(p, sr, si, sb);
        }
    }
    if (a.mode == 2) {
        rmax = warp_max_bits(rmax);
        xmax = warp_max_bits(xmax);
        __shared__ unsigned long long sm[2][8];
        if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = rmax; sm[1][threadIdx.x >> 5] = xmax; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { rmax = max(rmax, sm[0][w]); xmax = max(xmax, sm[1][w]); }
            a.part[s * 2 * gridDim.x + 2 * blockIdx.x] = __longlong_as_double((long long)rmax);
            a.part[s * 2 * gridDim.x + 2 * blockIdx.x + 1] = __longlong_as_double((long long)xmax);
        }
    }
}

// padded[s * np + p] = orig[s * n + slot2orig[p]] (0 on pad slots); shift = blockIdx.y
__global__ void k_gather(int64_t np, int64_t n, const int64_t *__restrict__ s2o, const double2 *__restrict__ orig,
                         double2 *__restrict__ padded) {
    const int64_t s = blockIdx.y;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = s2o[p];
        padded[s * np + p] = (o >= 0) ? orig[s * n + o] : mk(0.0, 0.0);
    }
}
__global__ void k_scatter(int64_t np, int64_t n, const int64_t *__restrict__ s2o, const double2 *__restrict__ padded,
                          double2 *__restrict__ orig) {
    const int64_t s = blockIdx.y;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = s2o[p];
        if (o >= 0) orig[s * n + o] = padded[s * np + p];
    }
}


template <typename C>
size_t tma_smem(int S, int nst, int chunk) {
    const int kCols = chunk / (kTileRows * (int)sizeof(C));
    const int nvec = ((S + kCols - 1) / kCols) * kCols;
    return (size_t)nst * chunk + 2 * (size_t)nst * sizeof(uint64_t) + 2 * (size_t)nvec * sizeof(C);
}

template <typename C>
void (*sweep_kernel(TmaVariant v))(const SweepTmaParams) {
    if (v.chunk == 8192)
        return v.cps == 2 ? k_sweep_tma<C, 2, 8192> : v.cps == 4 ? k_sweep_tma<C, 4, 8192> : k_sweep_tma<C, 3, 8192>;
    return v.cps == 2 ? k_sweep_tma<C, 2, 16384> : v.cps == 4 ? k_sweep_tma<C, 4, 16384> : k_sweep_tma<C, 3, 16384>;
}

// Sweep arguments of the plan's factors for `nshift` shifts starting at shift 0; the
// caller sets the vectors, counters and flags.
SweepArgs sweep_args(const kore_plan *p, int nshift) {
    SweepArgs a;
    a.K = p->K; a.S = p->S; a.nlev = p->nlev; a.nshift = nshift; a.levs = p->d_lev;
    a.Dinv = p->d_Dinv; a.G = p->d_Gm; a.H = p->d_Hm; a.LU = p->d_LU;
    a.f_stride = p->f_stride(); a.lu_stride = p->lu_stride();
    a.ell_col = p->d_ell_col; a.ell_val = p->d_ell_val; a.ell_w = p->ell_w; a.ell_stride = p->ell_stride();
    a.rscale = p->d_rscale;
    a.live_mask = ~0u;
    return a;
}

// Tensor maps, ring depth and the cooperative launch of the k_sweep_tma variant v (CTAs
// per SM, chunk bytes); the completion counters a.cnt are zeroed first.
template <typename C>
int launch_sweep(const kore_plan *p, const SweepArgs &a, cudaStream_t st, TmaVariant v = kTmaDefault) {
    SweepTmaParams P;
    P.a = a;
    const int rb = (int)sizeof(C) / 2;
    const int cps = v.cps;
    if (v.chunk != 8192 && v.chunk != 16384) return KORE_EINVAL;
    const int kCols = v.chunk / (kTileRows * (int)sizeof(C));
    const int ns = a.nshift;
    KORE_TRY(kore_encode_block_map(&P.maps[kMapDinv], p->d_Dinv, rb, p->S, p->K, ns, p->f_stride(), kTileRows, kCols));
    KORE_TRY(kore_encode_block_map(&P.maps[kMapG], p->d_Gm, rb, p->S, p->K, ns, p->f_stride(), kTileRows, kCols));
    KORE_TRY(kore_encode_block_map(&P.maps[kMapH], p->d_Hm, rb, p->S, p->K, ns, p->f_stride(), kTileRows, kCols));
    KORE_TRY(kore_encode_block_map(&P.maps[kMapLU], p->d_LU, rb, p->S, p->lu_mats, ns, p->lu_stride(), kTileRows,
                                   kCols));
    // ring depth: as many slots as fit cps CTAs in the SM's shared memory
    int smem_sm = 0, smem_blk = 0;
    KORE_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, p->device));
    KORE_CUDA_TRY(cudaDeviceGetAttribute(&smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device));
    void (*kern)(const SweepTmaParams) = sweep_kernel<C>(v);
    cudaFuncAttributes fa;
    KORE_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
    const size_t static_smem = fa.sharedSizeBytes + 1024;   // + the per-CTA reserve of the SM
    const size_t budget = std::min<size_t>((size_t)smem_sm / cps - static_smem,
                                           (size_t)smem_blk - fa.sharedSizeBytes);
    int nst = kMaxRing;
    while (nst > 2 && tma_smem<C>(p->S, nst, v.chunk) > budget) --nst;
    if (tma_smem<C>(p->S, nst, v.chunk) > budget) return KORE_EINVAL;
    P.nst = nst;
    const size_t smem = tma_smem<C>(p->S, nst, v.chunk);
    KORE_TRY(kore_allow_max_dyn_smem(kern, p->device));
    int occ = 0;
    KORE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTmaThreads, smem));
    if (occ < 1) return KORE_EINVAL;
    occ = std::min(occ, cps);
    KORE_CUDA_TRY(cudaMemsetAsync(a.cnt, 0, (size_t)ns * p->sweep_stages() * p->K * sizeof(int), st));
    void *args[] = {&P};
    dim3 grid(p->num_sms * occ), block(kTmaThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kern, grid, block, args, smem, st));
    KORE_LAUNCHED(1);
    return KORE_OK;
}

// Autotuner of the sweep's variant (CTAs per SM, chunk size), keyed on the plan's shape: the first
// non-accumulating sweep of a shape (padded block size, blocks, width of the level-0
// coupling rows, precision, shifts) times every variant on its own work (a
// non-accumulating sweep gives the same result each time it runs) and keeps the fastest
// for every later sweep of that shape in the process.
struct TuneKey {
    int S, K, ell_w, prec, nshift;
    bool operator<(const TuneKey &o) const {
        return std::tie(S, K, ell_w, prec, nshift) < std::tie(o.S, o.K, o.ell_w, o.prec, o.nshift);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, TmaVariant> g_tune;
TmaVariant g_force{0, 0};   // kore_sweep_variant: every sweep uses it instead of the autotuner's choice

template <typename C>
int tune_sweep(kore_plan *p, const SweepArgs &a, TmaVariant *best) {
    cudaEvent_t e0, e1;
    KORE_CUDA_TRY(cudaEventCreate(&e0));
    KORE_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    int rc = KORE_OK;
    *best = kTmaDefault;
    for (const TmaVariant v : kTmaVariants) {
        float ms = 0.f;
        for (int rep = 0; rep < 2 && rc == KORE_OK; ++rep) {   // the second run is timed
            if (cudaEventRecord(e0, p->stream) != cudaSuccess) rc = KORE_ECUDA;
            if (rc == KORE_OK) rc = launch_sweep<C>(p, a, p->stream, v);
            if (rc == KORE_OK && cudaEventRecord(e1, p->stream) != cudaSuccess) rc = KORE_ECUDA;
            if (rc == KORE_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = KORE_ECUDA;
            if (rc == KORE_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = KORE_ECUDA;
        }
        if (rc == KORE_EINVAL) { rc = KORE_OK; continue; }   // the variant does not fit this shape
        if (rc != KORE_OK) break;
        if (ms < best_ms) { best_ms = ms; *best = v; }
    }
    // the chosen variant runs last, so the sweep's outputs are its own
    if (rc == KORE_OK) rc = launch_sweep<C>(p, a, p->stream, *best);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate, const int *skip,
          unsigned live_mask) {
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, true));
    SweepArgs a = sweep_args(p, p->nshift);
    a.live_mask = live_mask;
    a.b = b; a.bnorm = bnorm;
    a.f = p->d_flo; a.z = p->d_zlo; a.x = p->d_xlo;
    a.out = x; a.accumulate = accumulate; a.cnt = p->d_cnt; a.err = p->d_err;
    a.skip = skip; a.skip_stride = (int)(sizeof(IrState) / sizeof(int));
    a.count = &p->d_ir->sweeps; a.count_total = &p->d_ir->sweeps_total;
    const bool fp64 = p->prec == KORE_PREC_FP64;
    const TuneKey key{p->S, p->K, p->ell_w, p->prec, p->nshift};
    TmaVariant v{0, 0};
    bool forced = false;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (g_force.cps != 0) { v = g_force; forced = true; }
        else if (it != g_tune.end()) v = it->second;
    }
    int s;
    if (v.cps == 0 && !accumulate && !forced) {
        s = fp64 ? tune_sweep<double2>(p, a, &v) : tune_sweep<float2>(p, a, &v);
        if (s == KORE_OK) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tune[key] = v;
        }
    } else {
        if (v.cps == 0) v = kTmaDefault;
        s = fp64 ? launch_sweep<double2>(p, a, p->stream, v) : launch_sweep<float2>(p, a, p->stream, v);
    }
    p->sweep_cps = v.cps;
    p->sweep_chunk = v.chunk;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, false));
    return s;
}

}  // namespace

extern "C" int kore_sweep_variant(int ctas_per_sm, int chunk_bytes) {
    bool ok = ctas_per_sm == 0 && chunk_bytes == 0;
    for (const TmaVariant v : kTmaVariants) ok = ok || (v.cps == ctas_per_sm && v.chunk == chunk_bytes);
    if (!ok) return KORE_EINVAL;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_force = TmaVariant{ctas_per_sm, chunk_bytes};
    return KORE_OK;
}

namespace {

unsigned absmax_grid(int64_t np) { return std::min<unsigned>(kore_div_up(np, 256), 1024u); }

// ||v_s||_inf of nshift padded vectors into out[s] (device); scratch: g * nshift doubles
int absmax(kore_plan *p, const double2 *v, double *out, double *scratch) {
    const unsigned g = absmax_grid(p->np);
    k_absmax<<<dim3(g, p->nshift), 256, 0, p->stream>>>(p->np, v, scratch);
    k_reduce_max<<<p->nshift, 1024, 0, p->stream>>>(scratch, (int)g, out);
    KORE_LAUNCHED(2);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

// CTAs of one sparse product: the 4-lane part, then 8 long rows per CTA
unsigned spmv_short_blocks(int64_t np) { return kore_div_up(np * kRowLanes, 256); }
unsigned spmv_grid(const kore_plan *p) { return spmv_short_blocks(p->np) + kore_div_up(p->nlong, 8); }
size_t spmv_smem(const kore_plan *p) { return (size_t)spmv_window(p->S) * sizeof(double2); }

SpmvArgs spmv_args(const kore_plan *p, int mode, const double2 *x, double2 *y) {
    SpmvArgs a;
    a.np = p->np; a.S = p->S; a.K = p->K; a.mode = mode; a.has_b = p->has_b ? 1 : 0;
    a.srow = p->d_srow; a.smid = p->d_smid; a.scol = p->d_scol; a.sval = p->d_sval;
    a.brow = p->d_brow; a.bcol = p->d_bcol; a.bval = p->d_bval;
    a.long_rows = p->d_long_rows; a.nlong = p->nlong; a.short_blocks = (int)spmv_short_blocks(p->np);
    a.lam = mk(0.0, 0.0); a.sig = nullptr;
    a.x = x; a.rhs = nullptr; a.y = y; a.part = nullptr;
    a.skip = nullptr; a.skip_stride = 0;
    a.live_mask = ~0u;
    return a;
}

}  // namespace

int kore_spmv_prepare(kore_plan *p) {
    // the x window of a CTA exceeds the default 48 KB of shared memory for S > 760
    return kore_allow_max_dyn_smem(k_spmv, p->device);
}

int kore_spmv_b(kore_plan *p, const double2 *x, double2 *y) {
    if (!p->has_b) return KORE_EINVAL;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
    k_spmv<<<spmv_grid(p), 256, spmv_smem(p), p->stream>>>(spmv_args(p, 0, x, y));
    KORE_LAUNCHED(1);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_b_shifts(kore_plan *p, const double2 *x, double2 *y, unsigned live_mask) {
    if (!p->has_b) return KORE_EINVAL;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
    SpmvArgs a = spmv_args(p, 0, x, y);
    a.live_mask = live_mask;
    k_spmv<<<dim3(spmv_grid(p), std::max(1, p->nshift)), 256, spmv_smem(p), p->stream>>>(a);
    KORE_LAUNCHED(1);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_a_shifts(kore_plan *p, const double2 *x, double2 *y, unsigned live_mask) {
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
    SpmvArgs a = spmv_args(p, 1, x, y);   // A x - 0 B x
    a.has_b = 0;
    a.live_mask = live_mask;
    k_spmv<<<dim3(spmv_grid(p), std::max(1, p->nshift)), 256, spmv_smem(p), p->stream>>>(a);
    KORE_LAUNCHED(1);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_pencil(kore_plan *p, double lre, double lim, const double2 *x, double2 *y) {
    SpmvArgs a = spmv_args(p, 1, x, y);
    a.lam = mk(lre, lim);
    k_spmv<<<spmv_grid(p), 256, spmv_smem(p), p->stream>>>(a);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_gather(kore_plan *p, const double2 *orig, double2 *padded) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_gather<<<grid, 256, 0, p->stream>>>(p->np, p->n, p->d_slot2orig, orig, padded);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_scatter(kore_plan *p, const double2 *padded, double2 *orig) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_scatter<<<grid, 256, 0, p->stream>>>(p->np, p->n, p->d_slot2orig, padded, orig);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_gather_shifts(kore_plan *p, const double2 *orig, double2 *padded) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_gather<<<dim3(grid, p->nshift), 256, 0, p->stream>>>(p->np, p->n, p->d_slot2orig, orig, padded);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_scatter_shifts(kore_plan *p, const double2 *padded, double2 *orig) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_scatter<<<dim3(grid, p->nshift), 256, 0, p->stream>>>(p->np, p->n, p->d_slot2orig, padded, orig);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

namespace {

// one thread per shift
__global__ void k_ir_begin(IrState *st, int nshift, unsigned live_mask) {
    const int s = threadIdx.x;
    if (s >= nshift) return;
    if (!mask_has(live_mask, s)) {   // not part of this application: nothing to refine
        st[s].done = 1;
        return;
    }
    st[s].done = 0;
    st[s].prev = 1e300;
    st[s].applies += 1;
}

// One CTA per shift s: eta = ||r||_inf / (||M||_inf ||x||_inf + ||b||_inf) from the
// per-CTA maxima of the residual kernel; stop when eta <= tol or when it no longer
// decreases (FP64 floor).
// Per-shift refinement tolerances of one application (shifts past 31 use the scalar).
struct ShiftTols {
    double t[32];
    int valid;
};

__global__ void k_ir_check(const double *__restrict__ part, int n, const double *__restrict__ bnorm,
                           const double *__restrict__ minf, double tol0, ShiftTols tols, IrState *stall, double *rn) {
    const int s = blockIdx.x;
    const double tol = (tols.valid && s < 32) ? tols.t[s] : tol0;
    IrState *st = stall + s;
    if (st->done) return;
    part += (int64_t)s * 2 * n;
    // maxima of non-negative doubles as bits (a NaN among them stays, and is caught below)
    unsigned long long rb = 0, xb = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        rb = max(rb, abs_bits(part[2 * i]));
        xb = max(xb, abs_bits(part[2 * i + 1]));
    }
    rb = warp_max_bits(rb);
    xb = warp_max_bits(xb);
    __shared__ unsigned long long s0[32], s1[32];
    if ((threadIdx.x & 31) == 0) { s0[threadIdx.x >> 5] = rb; s1[threadIdx.x >> 5] = xb; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { rb = max(rb, s0[w]); xb = max(xb, s1[w]); }
    const double rm = __longlong_as_double((long long)rb), xm = __longlong_as_double((long long)xb);
    const double den = minf[s] * xm + bnorm[s];
    // a NaN in r, x or b makes eta NaN (a NaN denominator must not read as converged)
    const double eta = (den == 0.0) ? 0.0 : rm / den;
    if (!(eta == eta)) {
        st->nan = 1;
        st->done = 1;
        return;
    }
    if (eta <= tol || eta > 0.9 * st->prev) {
        st->done = 1;
        st->eta_max = fmax(st->eta_max, eta);
        return;
    }
    st->prev = eta;
    st->iters += 1;
    st->iters_cur += 1;
    rn[s] = rm;
}

__global__ void k_ir_end(IrState *st, int nshift) {
    const int s = threadIdx.x;
    if (s >= nshift) return;
    if (st[s].iters_cur > st[s].iters_max) st[s].iters_max = st[s].iters_cur;
    // the loop ran out of corrections before the test passed: report the last measured
    // eta (taken before the final correction, so an upper estimate)
    if (!st[s].done && st[s].iters_cur > 0) st[s].eta_max = fmax(st[s].eta_max, st[s].prev);
    st[s].iters_cur = 0;
}

}  // namespace

// Mixed precision: the refinement loop runs without host synchronisation.  Its length
// is bounded (kIrMax corrections); each step is a residual kernel, a convergence check
// (one CTA per shift) and a correction sweep, and once the check marks a shift done
// the remaining work of that shift is skipped (kernels return at once when every
// shift is done).
constexpr int kIrMax = 6;
int kore_apply_inverse(kore_plan *p, const double2 *b, double2 *x, double tol, unsigned live_mask,
                       const double *shift_tols) {
    if (!p->factored) return KORE_ENOTFACTORED;
    double *bn = p->d_bn, *rn = p->d_rn;
    KORE_TRY(absmax(p, b, bn, p->d_part));
    if (p->prec != KORE_PREC_MIXED) return sweep(p, b, bn, x, 0, nullptr, live_mask);
    if (!(tol > 0.0)) tol = 1e-14;
    ShiftTols tols{};
    tols.valid = shift_tols ? 1 : 0;
    for (int s = 0; s < 32 && shift_tols && s < p->nshift; ++s) tols.t[s] = (shift_tols[s] > 0.0) ? shift_tols[s] : tol;
    const int ns = p->nshift;
    const int skip_stride = (int)(sizeof(IrState) / sizeof(int));
    k_ir_begin<<<1, ns, 0, p->stream>>>(p->d_ir, ns, live_mask);
    KORE_LAUNCHED(1);
    KORE_TRY(sweep(p, b, bn, x, 0, nullptr, live_mask));
    const unsigned grid = spmv_grid(p);
    SpmvArgs ra = spmv_args(p, 2, x, p->d_rb);
    ra.sig = p->d_sigma; ra.rhs = b; ra.part = p->d_part; ra.skip = &p->d_ir->done; ra.skip_stride = skip_stride;
    ra.live_mask = live_mask;
    for (int it = 0; it < kIrMax; ++it) {
        if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
        k_spmv<<<dim3(grid, ns), 256, spmv_smem(p), p->stream>>>(ra);
        k_ir_check<<<ns, 1024, 0, p->stream>>>(p->d_part, (int)grid, bn, p->d_minf, tol, tols, p->d_ir, rn);
        KORE_LAUNCHED(2);
        if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
        KORE_TRY(sweep(p, p->d_rb, rn, x, 1, &p->d_ir->done, live_mask));
    }
    k_ir_end<<<1, ns, 0, p->stream>>>(p->d_ir, ns);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_ir_reset(kore_plan *p) {
    // everything but the lifetime sweep counter of shift 0
    for (int s = 0; s < std::max(1, p->nshift); ++s)
        KORE_CUDA_TRY(cudaMemsetAsync(p->d_ir + s, 0, offsetof(IrState, sweeps_total), p->stream));
    return KORE_OK;
}

// Aggregate over the factorised shifts: sweep counts of shift 0 (every launch counts
// there), worst refinement count and eta, NaN in any shift.
int kore_ir_read(kore_plan *p, IrState *out) {
    const int ns = std::max(1, p->nshift);
    std::vector<IrState> all(ns);
    KORE_CUDA_TRY(cudaMemcpyAsync(all.data(), p->d_ir, ns * sizeof(IrState), cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    *out = all[0];
    for (int s = 1; s < ns; ++s) {
        out->nan |= all[s].nan;
        out->iters_max = std::max(out->iters_max, all[s].iters_max);
        out->eta_max = std::max(out->eta_max, all[s].eta_max);
        out->iters += all[s].iters;
    }
    return KORE_OK;
}

// ---------------------------------------------------------------------------------
// Allocation-free solve: kore_solve_dev_noalloc (include/kore_gpu.h).
//
// Some callers cannot allocate device memory at the moment they need a solve: code
// that runs under a fixed memory budget or a pool it does not own, code that must not
// trigger the implicit device synchronisation of cudaMalloc/cudaFree inside a
// latency-critical loop, or a host library that is handed only a stream.  For them the
// scratch of one solve (padded right-hand side and solution, the reduction vectors of
// the sweep, the FP64 residual and the per-CTA maxima of the refinement loop, the
// norm partials, the refinement state, the sweep's completion counters and the error
// flag) lives in the file-scope array below instead of in buffers of the plan or of a
// caller.  Its size
// is fixed at kNoAllocMaxNp padded unknowns (about 1.6 MB, held by every GPU that
// loads the library until the process exits); larger problems are rejected.
// The kernels are the ones of kore_solve_dev; only their scratch pointers differ.
namespace {

constexpr int64_t kNoAllocMaxNp = 16384;
constexpr int64_t kNoAllocMaxCnt = 32768;   // sweep completion counters: (3 levels + 2) x blocks
constexpr int64_t kNoAllocMaxSpmvCta = (kNoAllocMaxNp * kRowLanes + 255) / 256 + kNoAllocMaxNp / 8 + 1;

struct NoAllocScratch {
    double2 bp[kNoAllocMaxNp];      // padded right-hand side (complex128)
    double2 xp[kNoAllocMaxNp];      // padded solution
    double2 r[kNoAllocMaxNp];       // FP64 residual of the refinement loop
    double2 f[kNoAllocMaxNp];       // sweep reduction vectors, room for complex128
    double2 z[kNoAllocMaxNp];
    double2 x[kNoAllocMaxNp];
    double part[2 * kNoAllocMaxSpmvCta];   // per-CTA maxima of the residual kernel
    double red[2048 + 8];                  // ||b||_inf partials [0, 2048), then scalars
    IrState ir;
    int cnt[kNoAllocMaxCnt];              // sweep completion counters
    int err;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch, looked up once per device (the symbol's name
// in host code is only a stand-in and must never be passed to a kernel).
std::mutex g_noalloc_mu;
NoAllocScratch *g_noalloc_addr[64] = {};

int noalloc_scratch(int device, NoAllocScratch **out) {
    if (device < 0 || device >= 64) return KORE_EINVAL;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            std::fprintf(stderr, "kore: cudaGetSymbolAddress of the no-allocation scratch failed: %s\n",
                         cudaGetErrorString(e));
            return KORE_ECUDA;
        }
        g_noalloc_addr[device] = static_cast<NoAllocScratch *>(ptr);
    }
    *out = g_noalloc_addr[device];
    return KORE_OK;
}

template <typename C>
int noalloc_sweep(kore_plan *p, NoAllocScratch *s, const double2 *b, const double *bnorm, double2 *x, int accumulate,
                  const int *skip, cudaStream_t st) {
    SweepArgs a = sweep_args(p, 1);   // shift 0
    a.b = b; a.bnorm = bnorm;
    a.f = s->f; a.z = s->z; a.x = s->x;
    a.out = x; a.accumulate = accumulate; a.cnt = s->cnt; a.err = &s->err;
    a.skip = skip; a.skip_stride = 0; a.count = &s->ir.sweeps; a.count_total = &s->ir.sweeps_total;
    return launch_sweep<C>(p, a, st, p->sweep_cps > 0 ? TmaVariant{p->sweep_cps, p->sweep_chunk} : kTmaDefault);
}

int noalloc_solve(kore_plan *p, NoAllocScratch *s, const double2 *b_dev, double2 *x_dev, double tol, cudaStream_t st) {
    const bool mixed = p->prec == KORE_PREC_MIXED;
    const unsigned g = std::min<unsigned>(kore_div_up(p->np, 256), 1024u);
    double *bn = s->red + 2048, *rn = s->red + 2049;
    // every call starts from a cleared error flag and refinement state
    KORE_CUDA_TRY(cudaMemsetAsync(&s->err, 0, sizeof(int), st));
    KORE_CUDA_TRY(cudaMemsetAsync(&s->ir, 0, sizeof(IrState), st));
    k_gather<<<std::min<unsigned>(kore_div_up(p->np, 256), 2048u), 256, 0, st>>>(p->np, p->n, p->d_slot2orig, b_dev,
                                                                                 s->bp);
    k_absmax<<<g, 256, 0, st>>>(p->np, s->bp, s->red);
    k_reduce_max<<<1, 1024, 0, st>>>(s->red, (int)g, bn);
    KORE_LAUNCHED(3);
    if (!mixed) {
        KORE_TRY(noalloc_sweep<double2>(p, s, s->bp, bn, s->xp, 0, nullptr, st));
    } else {
        if (!(tol > 0.0)) tol = 1e-14;
        k_ir_begin<<<1, 1, 0, st>>>(&s->ir, 1, ~0u);
        KORE_LAUNCHED(1);
        KORE_TRY(noalloc_sweep<float2>(p, s, s->bp, bn, s->xp, 0, nullptr, st));
        const unsigned grid = spmv_grid(p);
        SpmvArgs ra = spmv_args(p, 2, s->xp, s->r);
        ra.lam = mk(p->sigma_re, p->sigma_im); ra.rhs = s->bp; ra.part = s->part; ra.skip = &s->ir.done;
        for (int it = 0; it < kIrMax; ++it) {
            k_spmv<<<grid, 256, spmv_smem(p), st>>>(ra);
            k_ir_check<<<1, 1024, 0, st>>>(s->part, (int)grid, bn, p->d_minf, tol, ShiftTols{}, &s->ir, rn);
            KORE_LAUNCHED(2);
            KORE_TRY(noalloc_sweep<float2>(p, s, s->r, rn, s->xp, 1, &s->ir.done, st));
        }
    }
    k_scatter<<<std::min<unsigned>(kore_div_up(p->np, 256), 2048u), 256, 0, st>>>(p->np, p->n, p->d_slot2orig, s->xp,
                                                                                  x_dev);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

}  // namespace

extern "C" int kore_solve_dev_noalloc(kore_plan *p, const void *b_dev, void *x_dev, double refine_tol, void *stream) {
    if (!p || !b_dev || !x_dev) return KORE_EINVAL;
    if (p->np > kNoAllocMaxNp || (int64_t)p->sweep_stages() * p->K > kNoAllocMaxCnt) {
        std::fprintf(stderr,
                     "kore_solve_dev_noalloc: %lld padded unknowns in %d blocks exceed the fixed scratch "
                     "(%lld unknowns, %lld block counters); use kore_solve_dev\n",
                     (long long)p->np, p->K, (long long)kNoAllocMaxNp, (long long)kNoAllocMaxCnt);
        return KORE_EINVAL;
    }
    if (!p->factored) return KORE_ENOTFACTORED;
    if (p->nshift != 1) {
        std::fprintf(stderr, "kore_solve_dev_noalloc: the plan holds %d factorised shifts; this entry point "
                             "solves with a plan of one shift (kore_factor)\n", p->nshift);
        return KORE_EINVAL;
    }
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != p->device) KORE_CUDA_TRY(cudaSetDevice(p->device));
    NoAllocScratch *s = nullptr;
    int rc = noalloc_scratch(p->device, &s);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (rc == KORE_OK) rc = noalloc_solve(p, s, static_cast<const double2 *>(b_dev), static_cast<double2 *>(x_dev),
                                          refine_tol, st);
    if (rc == KORE_OK) {
        // wait for this call's kernels, then read its error flag and NaN state
        int flags[2] = {0, 0};
        if (cudaMemcpyAsync(&flags[0], &s->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(&flags[1], &s->ir.nan, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = KORE_ECUDA;
        else if (flags[0] != 0)
            rc = KORE_ETIMEOUT;
        else if (flags[1] != 0)
            rc = KORE_ENAN;
    }
    if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
    return rc;
}
