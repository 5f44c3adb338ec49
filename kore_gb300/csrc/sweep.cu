// Solves with the block-cyclic-reduction factors of factor.cu, sparse products and
// the FP64 refinement loop.
//
// (A - sigma B) x = b with row scaling R and s = ||b||_inf (keeps complex64 in range):
// the right-hand side c = s^-1 R b is reduced level by level exactly as the blocks were,
//     level l, odd blocks j:   z_j = D_j^-1 f_j
//     level l, even blocks i:  f_i <- f_i - L_i z_jl - U_i z_jr        (CSR couplings at level 0)
// the last block is solved, x_0 = D_0^-1 f_0, and the levels are unwound in reverse,
//     level l, odd blocks j:   x_j = z_j - G_j x_jl - H_j x_jr,
// then x <- s x.  One cooperative persistent kernel runs all phases (about 3 log2 K of
// them) with a bounded grid barrier between dependent phases; inside a phase every
// (block, row tile) is independent, so each phase is a batched matrix-vector product
// streaming the factors from HBM across the whole GPU.
//
// Every kernel here works on all factorised shifts at once (shift s: its own factors,
// row scales and vectors at offset s * stride), so a batch of forcing frequencies is
// one sweep launch.
//
// In mixed precision the factors are complex64 and the result is refined in FP64:
//     r = b - (A - sigma B) x,  x += M32^-1 r   until ||r||_inf <= tol (||M||_inf ||x||_inf + ||b||_inf).
#include "kore_internal.cuh"
#include <cstddef>
#include <mutex>

namespace {

constexpr int kSweepWarps = 8;                 // warps of a sweep CTA; they split the columns
constexpr int kSweepThreads = 32 * kSweepWarps;  // a CTA computes 32 rows of one block

__device__ __forceinline__ double2 ldcg(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2 *p) { return __ldcg(p); }
__device__ __forceinline__ void stcg(double2 *p, double2 v) { __stcg(p, v); }
__device__ __forceinline__ void stcg(float2 *p, float2 v) { __stcg(p, v); }

// Rows [r0, r0+32) of M1 v1 (+ M2 v2): lane = row, warp w = column range; column-major
// S x S blocks so every column read is a coalesced 32-row segment.  The partial sums
// of the warps are combined through shared memory; the result is returned to the
// lanes of warp 0 (row r0 + lane).
template <typename C, int U>
__device__ __forceinline__ void col_range_dot(const C *__restrict__ M1, const C *__restrict__ v1,
                                              const C *__restrict__ M2, const C *__restrict__ v2, int S, int r,
                                              int c0, int c1, C &a0, C &a1) {
    int c = c0;
    for (; c + U <= c1; c += U) {
        C m[U], n[U];
#pragma unroll
        for (int t = 0; t < U; ++t) m[t] = __ldg(M1 + r + (int64_t)(c + t) * S);
        if (M2) {
#pragma unroll
            for (int t = 0; t < U; ++t) n[t] = __ldg(M2 + r + (int64_t)(c + t) * S);
        }
#pragma unroll
        for (int t = 0; t < U; ++t) a0 = cfma(a0, m[t], v1[c + t]);
        if (M2) {
#pragma unroll
            for (int t = 0; t < U; ++t) a1 = cfma(a1, n[t], v2[c + t]);
        }
    }
    for (; c < c1; ++c) {
        a0 = cfma(a0, __ldg(M1 + r + (int64_t)c * S), v1[c]);
        if (M2) a1 = cfma(a1, __ldg(M2 + r + (int64_t)c * S), v2[c]);
    }
}

// Rows [r0, r0+32) of M1 v1 (+ M2 v2): lane = row, warp w = column range; column-major
// S x S blocks so every column read is a coalesced 32-row segment.  Eight loads are in
// flight per thread (8 of one matrix, or 4 + 4 of two).  The partial sums of the warps
// are combined through shared memory; the result is returned to the lanes of warp 0
// (row r0 + lane).
template <typename C>
__device__ __forceinline__ C tile_gemv(const C *__restrict__ M1, const C *__restrict__ v1, const C *__restrict__ M2,
                                       const C *__restrict__ v2, int S, int r0, C (*red)[33]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r = r0 + lane;
    const int cw = (S + kSweepWarps - 1) / kSweepWarps;
    const int c0 = w * cw, c1 = min(S, c0 + cw);
    C a0 = czero<C>(), a1 = czero<C>();
    if (r < S) {
        if (M2) col_range_dot<C, 4>(M1, v1, M2, v2, S, r, c0, c1, a0, a1);
        else col_range_dot<C, 8>(M1, v1, nullptr, nullptr, S, r, c0, c1, a0, a1);
    }
    red[w][lane] = a0 + a1;
    __syncthreads();
    C out = czero<C>();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < kSweepWarps; ++k) out = out + red[k][lane];
    }
    return out;
}

struct SweepArgs {
    int K, S, nlev, nshift;
    const BcrLevel *levs;
    const void *Dinv, *G, *H, *LU;
    int64_t f_stride, lu_stride;     // per-shift strides of the factor blocks (elements)
    const int *arow, *acol, *asplit;
    const double2 *aval;
    const double2 *b;                // nshift x np right-hand sides (complex128, padded)
    const double *rscale;            // nshift x np
    const double *bnorm;             // nshift scalings
    void *f, *z, *x;                 // nshift x np reduction vectors (factor precision)
    double2 *out;                    // nshift x np
    int accumulate;
    int *cnt;                        // completion counters: nshift x (3 nlev + 1) x K, zeroed before the launch
    int *err;
    const int *skip;                 // shift s is skipped when skip[s * skip_stride] != 0
    int skip_stride;
    int *count;                      // sweeps that ran
    int *count_total;
};

constexpr int kMaxLevels = 24;

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

// Dataflow sweep.  The tiles (32 rows of one block) of all stages are numbered in a
// topological order
//     A_0, B_0, A_1, B_1, ..., A_{L-1}, B_{L-1}, top, C_{L-1}, ..., C_0
// (A: z_j = D_j^-1 f_j, B: f_i -= L_i z_jl + U_i z_jr, C: x_j = z_j - G_j x_jl - H_j x_jr)
// and CTA c takes tiles c, c + G, c + 2G, ...  A tile waits only for the counters of
// the blocks it reads (e.g. a B tile for A of its two neighbours), and after writing
// its rows it adds 1 to the counter of (stage, block).  Tiles are taken in increasing
// order by co-resident CTAs, so every wait is on a tile of a lower number that some
// CTA is processing or has processed: no deadlock, and adjacent stages overlap.
template <typename C>
__global__ void __launch_bounds__(kSweepThreads, 3) k_sweep(SweepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *v1 = reinterpret_cast<C *>(smem_raw);
    C *v2 = v1 + a.S;
    __shared__ C red[kSweepWarps][33];
    __shared__ BcrLevel lv_s[kMaxLevels];
    __shared__ int64_t st_begin[3 * kMaxLevels + 2];
    // uniform over the grid: the flags were set by an earlier kernel
    if (a.skip) {
        bool all = true;
        for (int s = 0; s < a.nshift; ++s) all = all && (a.skip[s * a.skip_stride] != 0);
        if (all) return;
    }
    if (a.count && blockIdx.x == 0 && threadIdx.x == 0) { atomicAdd(a.count, 1); atomicAdd(a.count_total, 1); }
    const int S = a.S, ns = a.nshift, L = a.nlev, K = a.K;
    const int64_t SS = (int64_t)S * S, np = (int64_t)K * S;
    const int ntile = (S + 31) / 32;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nstage = 3 * L + 1;
    if (tid < L) lv_s[tid] = a.levs[tid];
    __syncthreads();
    // stage k: 0..2L-1 -> A_{k/2} (even k) / B_{k/2} (odd k); 2L -> top; 2L+1+m -> C_{L-1-m}
    if (tid == 0) {
        int64_t acc = 0;
        for (int k = 0; k < nstage; ++k) {
            st_begin[k] = acc;
            int nblk;
            if (k < 2 * L) nblk = (k & 1) ? lv_s[k >> 1].neven : lv_s[k >> 1].nodd;
            else if (k == 2 * L) nblk = 1;
            else nblk = lv_s[L - 1 - (k - 2 * L - 1)].nodd;
            acc += (int64_t)nblk * ntile * ns;
        }
        st_begin[nstage] = acc;
    }
    __syncthreads();
    const int64_t total = st_begin[nstage];
    // counter of (shift, stage id, block); stage ids: A_l = l, B_l = L + l, top = 2L, C_l = 2L + 1 + l
    auto ctr = [&](int64_t s, int sid, int64_t blk) -> int * { return a.cnt + ((s * nstage + sid) * K + blk); };
    auto live = [&](int64_t s) -> bool { return !(a.skip && a.skip[s * a.skip_stride] != 0); };
    auto fac = [&](const void *base, int64_t s) -> const C * { return static_cast<const C *>(base) + s * a.f_stride; };
    auto vec = [&](void *base, int64_t s) -> C * { return static_cast<C *>(base) + s * np; };
    auto rhs0 = [&](int64_t s, int64_t p) -> C {
        const double bn = a.bnorm[s];
        const double bscale = (bn > 0.0) ? 1.0 / bn : 1.0;
        return from_c128<C>((a.rscale[s * np + p] * bscale) * a.b[s * np + p]);
    };
    auto emit = [&](int64_t s, int64_t p, C val) {
        stcg(vec(a.x, s) + p, val);
        const double bn = a.bnorm[s];
        const double2 d = ((bn > 0.0) ? bn : 1.0) * to_c128(val);
        double2 *o = a.out + s * np + p;
        *o = a.accumulate ? *o + d : d;
    };
    // x of block b is final after C of the level that eliminated it (top for block 0)
    auto xready = [&](int64_t s, int64_t blk) -> int * {
        if (blk == 0) return ctr(s, 2 * L, 0);
        const int lb = __ffsll(blk) - 1;   // block b is odd at level ctz(b)
        return ctr(s, 2 * L + 1 + lb, blk);
    };

    int k = 0;
    for (int64_t g = blockIdx.x; g < total; g += gridDim.x) {
        while (g >= st_begin[k + 1]) ++k;
        const int64_t loc = g - st_begin[k];
        int kind, l;
        if (k < 2 * L) { kind = (k & 1) ? 1 : 0; l = k >> 1; }
        else if (k == 2 * L) { kind = 2; l = L; }
        else { kind = 3; l = L - 1 - (k - 2 * L - 1); }
        const int nblk = (kind == 0 || kind == 3) ? lv_s[l].nodd : (kind == 1 ? lv_s[l].neven : 1);
        const int64_t s = loc / ((int64_t)nblk * ntile);
        const int64_t rem = loc - s * nblk * ntile;
        const int64_t bi = rem / ntile;
        const int r0 = (int)(rem - bi * ntile) * 32;
        const bool go = live(s);
        int *done = nullptr;
        __syncthreads();   // shared vectors of the previous tile are no longer read
        if (kind == 0) {
            // ---------------------------------------------- A_l: z_j = Dinv_j f_j
            const BcrLevel lv = lv_s[l];
            const int64_t j = (2 * bi + 1) * lv.stride;
            done = ctr(s, l, j);
            if (go) {
                if (l > 0 && tid == 0) wait_count(ctr(s, L + l - 1, j), ntile, a.err);   // f_j from B_{l-1}
                __syncthreads();
                const C *f = vec(a.f, s);
                for (int c = tid; c < S; c += blockDim.x) v1[c] = (l == 0) ? rhs0(s, j * S + c) : ldcg(f + j * S + c);
                __syncthreads();
                const C val = tile_gemv<C>(fac(a.Dinv, s) + j * SS, v1, nullptr, nullptr, S, r0, red);
                if (w == 0 && r0 + lane < S) stcg(vec(a.z, s) + j * S + r0 + lane, val);
            }
        } else if (kind == 1) {
            // ---------------------------------------------- B_l: f_i -= L_i z_jl + U_i z_jr
            const BcrLevel lv = lv_s[l];
            const int64_t q = 2 * bi, i = q * lv.stride;
            const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
            const int64_t jl = (q - 1) * lv.stride, jr = (q + 1) * lv.stride;
            done = ctr(s, L + l, i);
            if (go) {
                if (tid == 0) {
                    if (hasl) wait_count(ctr(s, l, jl), ntile, a.err);
                    if (hasr) wait_count(ctr(s, l, jr), ntile, a.err);
                    if (l > 0) wait_count(ctr(s, L + l - 1, i), ntile, a.err);   // f_i from B_{l-1}
                }
                __syncthreads();
                const C *z = vec(a.z, s);
                C *f = vec(a.f, s);
                if (l == 0) {
                    // couplings from the CSR: warp w handles rows r0 + 4w .. r0 + 4w + 3
                    for (int rr = 0; rr < 4; ++rr) {
                        const int r = r0 + 4 * w + rr;
                        if (r >= S) break;
                        const int64_t p = i * S + r;
                        const double rs = a.rscale[s * np + p];
                        C acc = czero<C>();
                        if (hasl)
                            for (int e = a.arow[p] + lane; e < a.asplit[2 * p]; e += 32)
                                acc = cfma(acc, from_c128<C>(rs * a.aval[e]), ldcg(z + a.acol[e]));
                        if (hasr)
                            for (int e = a.asplit[2 * p + 1] + lane; e < a.arow[p + 1]; e += 32)
                                acc = cfma(acc, from_c128<C>(rs * a.aval[e]), ldcg(z + a.acol[e]));
                        acc = warp_sum(acc);
                        if (lane == 0) stcg(f + p, rhs0(s, p) - acc);
                    }
                } else {
                    const C *LU = static_cast<const C *>(a.LU) + s * a.lu_stride;
                    for (int c = tid; c < S; c += blockDim.x) {
                        v1[c] = hasl ? ldcg(z + jl * S + c) : czero<C>();
                        v2[c] = hasr ? ldcg(z + jr * S + c) : czero<C>();
                    }
                    __syncthreads();
                    const C *M1 = hasl ? LU + (lv.lu_L + q) * SS : (hasr ? LU + (lv.lu_U + q) * SS : nullptr);
                    const C *V1 = hasl ? v1 : v2;
                    const C *M2 = (hasl && hasr) ? LU + (lv.lu_U + q) * SS : nullptr;
                    C acc = czero<C>();
                    if (M1) acc = tile_gemv<C>(M1, V1, M2, v2, S, r0, red);
                    if (w == 0 && r0 + lane < S) {
                        const int64_t p = i * S + r0 + lane;
                        stcg(f + p, ldcg(f + p) - acc);
                    }
                }
            }
        } else if (kind == 2) {
            // ---------------------------------------------- top: x_0 = Dinv_0 f_0
            done = ctr(s, 2 * L, 0);
            if (go) {
                if (L > 0 && tid == 0) wait_count(ctr(s, 2 * L - 1, 0), ntile, a.err);   // f_0 from B_{L-1}
                __syncthreads();
                const C *f = vec(a.f, s);
                for (int c = tid; c < S; c += blockDim.x) v1[c] = (L == 0) ? rhs0(s, c) : ldcg(f + c);
                __syncthreads();
                const C val = tile_gemv<C>(fac(a.Dinv, s), v1, nullptr, nullptr, S, r0, red);
                if (w == 0 && r0 + lane < S) emit(s, r0 + lane, val);
            }
        } else {
            // ---------------------------------------------- C_l: x_j = z_j - G_j x_jl - H_j x_jr
            const BcrLevel lv = lv_s[l];
            const int64_t q = 2 * bi + 1, j = q * lv.stride;
            const bool hasr = q + 1 < lv.Kl;
            const int64_t jl = j - lv.stride, jr = j + lv.stride;
            done = ctr(s, 2 * L + 1 + l, j);
            if (go) {
                if (tid == 0) {
                    wait_count(xready(s, jl), ntile, a.err);
                    if (hasr) wait_count(xready(s, jr), ntile, a.err);
                }
                __syncthreads();
                const C *x = vec(a.x, s), *z = vec(a.z, s);
                for (int c = tid; c < S; c += blockDim.x) {
                    v1[c] = ldcg(x + jl * S + c);
                    v2[c] = hasr ? ldcg(x + jr * S + c) : czero<C>();
                }
                __syncthreads();
                const C acc = tile_gemv<C>(fac(a.G, s) + j * SS, v1, hasr ? fac(a.H, s) + j * SS : nullptr, v2, S,
                                           r0, red);
                if (w == 0 && r0 + lane < S) {
                    const int64_t p = j * S + r0 + lane;
                    emit(s, p, ldcg(z + p) - acc);
                }
            }
        }
        // publish: every write of the tile happens before the counter increment
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(done, 1);
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

// 4 lanes per row (measured fastest on this structure: each lane keeps ~10 independent
// gathers in flight), grid-stride over the rows; shift = blockIdx.y (vectors at s * np).
// mode 0: y = B x.  mode 1: y = A x - lam B x.  mode 2: y = b - (A x - lam B x), and
// per-CTA maxima of |y| and |x| into part[s * 2 gridDim.x + 2 blockIdx.x (+1)].
// lam = sig[s] when sig is given.
constexpr int kRowLanes = 4;
__global__ void __launch_bounds__(256) k_spmv(int64_t np, int mode, const int *__restrict__ arow,
                                              const int *__restrict__ acol, const double2 *__restrict__ aval,
                                              const int *__restrict__ brow, const int *__restrict__ bcol,
                                              const double *__restrict__ bval, int has_b, double lre, double lim,
                                              const double2 *__restrict__ sig, const double2 *__restrict__ x,
                                              const double2 *__restrict__ rhs, double2 *__restrict__ y,
                                              double *__restrict__ part, const int *__restrict__ skip,
                                              int skip_stride) {
    const int64_t s = blockIdx.y;
    if (skip && skip[s * skip_stride]) return;
    x += s * np;
    y += s * np;
    if (rhs) rhs += s * np;
    const int sub = threadIdx.x & (kRowLanes - 1);
    const int64_t row0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kRowLanes;
    const int64_t rstride = ((int64_t)gridDim.x * blockDim.x) / kRowLanes;
    const int64_t nrow_iter = (np + rstride - 1) / rstride;   // same trip count for every lane
    const double2 lam = sig ? sig[s] : mk(lre, lim);
    double rmax = 0.0, xmax = 0.0;
    for (int64_t t = 0; t < nrow_iter; ++t) {
        const int64_t p = row0 + t * rstride;
        const bool live = p < np;
        double2 sa = mk(0.0, 0.0), sb = mk(0.0, 0.0);
        if (live) {
            if (mode != 0) {
                const int e1 = arow[p + 1];
                for (int e = arow[p] + sub; e < e1; e += kRowLanes)
                    sa = cfma(sa, __ldg(aval + e), __ldg(x + __ldg(acol + e)));
            }
            if (has_b) {
                const int e1 = brow[p + 1];
                for (int e = brow[p] + sub; e < e1; e += kRowLanes) sb = sb + __ldg(bval + e) * __ldg(x + __ldg(bcol + e));
            }
        }
#pragma unroll
        for (int o = kRowLanes / 2; o > 0; o >>= 1) {
            sa.x += __shfl_down_sync(0xffffffffu, sa.x, o, kRowLanes);
            sa.y += __shfl_down_sync(0xffffffffu, sa.y, o, kRowLanes);
            sb.x += __shfl_down_sync(0xffffffffu, sb.x, o, kRowLanes);
            sb.y += __shfl_down_sync(0xffffffffu, sb.y, o, kRowLanes);
        }
        if (live && sub == 0) {
            double2 v = (mode == 0) ? sb : sa - lam * sb;
            if (mode == 2) {
                v = rhs[p] - v;
                rmax = fmax(rmax, fmax(fabs(v.x), fabs(v.y)));
                xmax = fmax(xmax, fmax(fabs(x[p].x), fabs(x[p].y)));
            }
            y[p] = v;
        }
    }
    if (mode == 2) {
        rmax = warp_max_d(rmax);
        xmax = warp_max_d(xmax);
        __shared__ double sm[2][8];
        if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = rmax; sm[1][threadIdx.x >> 5] = xmax; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { rmax = fmax(rmax, sm[0][w]); xmax = fmax(xmax, sm[1][w]); }
            part[s * 2 * gridDim.x + 2 * blockIdx.x] = rmax;
            part[s * 2 * gridDim.x + 2 * blockIdx.x + 1] = xmax;
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
int occupancy(kore_plan *p, size_t smem) {
    const int ti = (sizeof(C) == 16) ? 1 : 0;
    if (p->sweep_occ[ti] == 0) {
        auto kern = k_sweep<C>;
        if (smem > 48 * 1024)
            KORE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0;
        KORE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kSweepThreads, smem));
        p->sweep_occ[ti] = std::max(1, std::min(occ, 4));
    }
    return KORE_OK;
}

template <typename C>
int launch_sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate, const int *skip) {
    SweepArgs a;
    a.K = p->K; a.S = p->S; a.nlev = p->nlev; a.nshift = p->nshift; a.levs = p->d_lev;
    a.Dinv = p->d_Dinv; a.G = p->d_Gm; a.H = p->d_Hm; a.LU = p->d_LU;
    a.f_stride = p->f_stride(); a.lu_stride = p->lu_stride();
    a.arow = p->d_arow; a.acol = p->d_acol; a.asplit = p->d_asplit; a.aval = p->d_aval;
    a.b = b; a.rscale = p->d_rscale; a.bnorm = bnorm;
    a.f = p->d_flo; a.z = p->d_zlo; a.x = p->d_xlo;
    a.out = x; a.accumulate = accumulate; a.cnt = p->d_cnt; a.err = p->d_err;
    a.skip = skip; a.skip_stride = (int)(sizeof(IrState) / sizeof(int));
    a.count = &p->d_ir->sweeps; a.count_total = &p->d_ir->sweeps_total;
    const size_t smem = 2 * (size_t)p->S * sizeof(C);
    KORE_TRY(occupancy<C>(p, smem));
    const int occ = p->sweep_occ[sizeof(C) == 16 ? 1 : 0];
    KORE_CUDA_TRY(cudaMemsetAsync(p->d_cnt, 0, (size_t)p->nshift * (3 * p->nlev + 1) * p->K * sizeof(int), p->stream));
    void *args[] = {&a};
    dim3 grid(p->num_sms * occ), block(kSweepThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_sweep<C>, grid, block, args, smem, p->stream));
    KORE_LAUNCHED(1);
    return KORE_OK;
}

int sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate, const int *skip) {
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, true));
    const int s = (p->prec == KORE_PREC_FP64) ? launch_sweep<double2>(p, b, bnorm, x, accumulate, skip)
                                              : launch_sweep<float2>(p, b, bnorm, x, accumulate, skip);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, false));
    return s;
}

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

unsigned spmv_grid(int64_t np) { return kore_div_up(np * kRowLanes, 256); }

}  // namespace

int kore_spmv_b(kore_plan *p, const double2 *x, double2 *y) {
    if (!p->has_b) return KORE_EINVAL;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
    k_spmv<<<spmv_grid(p->np), 256, 0, p->stream>>>(p->np, 0, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                     p->d_bval, 1, 0.0, 0.0, nullptr, x, nullptr, y, nullptr, nullptr, 0);
    KORE_LAUNCHED(1);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_pencil(kore_plan *p, double lre, double lim, const double2 *x, double2 *y) {
    k_spmv<<<spmv_grid(p->np), 256, 0, p->stream>>>(p->np, 1, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                     p->d_bval, p->has_b ? 1 : 0, lre, lim, nullptr, x, nullptr, y,
                                                     nullptr, nullptr, 0);
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
__global__ void k_ir_begin(IrState *st, int nshift) {
    const int s = threadIdx.x;
    if (s >= nshift) return;
    st[s].done = 0;
    st[s].prev = 1e300;
    st[s].applies += 1;
}

// One CTA per shift s: eta = ||r||_inf / (||M||_inf ||x||_inf + ||b||_inf) from the
// per-CTA maxima of the residual kernel; stop when eta <= tol or when it no longer
// decreases (FP64 floor).
__global__ void k_ir_check(const double *__restrict__ part, int n, const double *__restrict__ bnorm,
                           const double *__restrict__ minf, double tol, IrState *stall, double *rn) {
    const int s = blockIdx.x;
    IrState *st = stall + s;
    if (st->done) return;
    part += (int64_t)s * 2 * n;
    double rm = 0.0, xm = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        rm = fmax(rm, part[2 * i]);
        xm = fmax(xm, part[2 * i + 1]);
    }
    rm = warp_max_d(rm);
    xm = warp_max_d(xm);
    __shared__ double s0[32], s1[32];
    if ((threadIdx.x & 31) == 0) { s0[threadIdx.x >> 5] = rm; s1[threadIdx.x >> 5] = xm; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { rm = fmax(rm, s0[w]); xm = fmax(xm, s1[w]); }
    const double den = minf[s] * xm + bnorm[s];
    const double eta = (den > 0.0) ? rm / den : 0.0;
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
    st[s].iters_cur = 0;
}

}  // namespace

// Mixed precision: the refinement loop runs without host synchronisation.  Its length
// is bounded (kIrMax corrections); each step is a residual kernel, a convergence check
// (one CTA per shift) and a correction sweep, and once the check marks a shift done
// the remaining work of that shift is skipped (kernels return at once when every
// shift is done).
constexpr int kIrMax = 6;
int kore_apply_inverse(kore_plan *p, const double2 *b, double2 *x, double tol) {
    if (!p->factored) return KORE_ENOTFACTORED;
    double *bn = p->d_bn, *rn = p->d_rn;
    KORE_TRY(absmax(p, b, bn, p->d_part));
    if (p->prec != KORE_PREC_MIXED) return sweep(p, b, bn, x, 0, nullptr);
    if (!(tol > 0.0)) tol = 1e-14;
    const int ns = p->nshift;
    const int skip_stride = (int)(sizeof(IrState) / sizeof(int));
    k_ir_begin<<<1, ns, 0, p->stream>>>(p->d_ir, ns);
    KORE_LAUNCHED(1);
    KORE_TRY(sweep(p, b, bn, x, 0, nullptr));
    const unsigned grid = spmv_grid(p->np);
    for (int it = 0; it < kIrMax; ++it) {
        if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
        k_spmv<<<dim3(grid, ns), 256, 0, p->stream>>>(p->np, 2, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                      p->d_bval, p->has_b ? 1 : 0, 0.0, 0.0, p->d_sigma, x, b, p->d_rb,
                                                      p->d_part, &p->d_ir->done, skip_stride);
        k_ir_check<<<ns, 1024, 0, p->stream>>>(p->d_part, (int)grid, bn, p->d_minf, tol, p->d_ir, rn);
        KORE_LAUNCHED(2);
        if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
        KORE_TRY(sweep(p, p->d_rb, rn, x, 1, &p->d_ir->done));
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
// grid-barrier counter, the error flag and the refinement state) lives in the
// file-scope array below instead of in buffers of the plan or of a caller.  Its size
// is fixed at kNoAllocMaxNp padded unknowns (about 1.6 MB, held by every GPU that
// loads the library until the process exits); larger problems are rejected.
// The kernels are the ones of kore_solve_dev; only their scratch pointers differ.
namespace {

constexpr int64_t kNoAllocMaxNp = 16384;
constexpr int64_t kNoAllocMaxCnt = 32768;   // sweep completion counters: (3 levels + 1) x blocks
constexpr int64_t kNoAllocMaxSpmvCta = (kNoAllocMaxNp * kRowLanes + 255) / 256;

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
    SweepArgs a;
    a.K = p->K; a.S = p->S; a.nlev = p->nlev; a.nshift = 1; a.levs = p->d_lev;
    a.Dinv = p->d_Dinv; a.G = p->d_Gm; a.H = p->d_Hm; a.LU = p->d_LU;   // shift 0
    a.f_stride = p->f_stride(); a.lu_stride = p->lu_stride();
    a.arow = p->d_arow; a.acol = p->d_acol; a.asplit = p->d_asplit; a.aval = p->d_aval;
    a.b = b; a.rscale = p->d_rscale; a.bnorm = bnorm;
    a.f = s->f; a.z = s->z; a.x = s->x;
    a.out = x; a.accumulate = accumulate; a.cnt = s->cnt; a.err = &s->err;
    a.skip = skip; a.skip_stride = 0; a.count = &s->ir.sweeps; a.count_total = &s->ir.sweeps_total;
    const size_t smem = 2 * (size_t)p->S * sizeof(C);
    auto kern = k_sweep<C>;
    if (smem > 48 * 1024)
        KORE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    KORE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kSweepThreads, smem));
    occ = std::max(1, std::min(occ, 4));
    KORE_CUDA_TRY(cudaMemsetAsync(s->cnt, 0, (size_t)(3 * p->nlev + 1) * p->K * sizeof(int), st));
    void *args[] = {&a};
    dim3 grid(p->num_sms * occ), block(kSweepThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kern, grid, block, args, smem, st));
    KORE_LAUNCHED(1);
    return KORE_OK;
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
        k_ir_begin<<<1, 1, 0, st>>>(&s->ir, 1);
        KORE_LAUNCHED(1);
        KORE_TRY(noalloc_sweep<float2>(p, s, s->bp, bn, s->xp, 0, nullptr, st));
        const unsigned grid = kore_div_up(p->np * kRowLanes, 256);
        for (int it = 0; it < kIrMax; ++it) {
            k_spmv<<<grid, 256, 0, st>>>(p->np, 2, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol, p->d_bval,
                                         p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, nullptr, s->xp, s->bp, s->r,
                                         s->part, &s->ir.done, 0);
            k_ir_check<<<1, 1024, 0, st>>>(s->part, (int)grid, bn, p->d_minf, tol, &s->ir, rn);
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
    if (p->np > kNoAllocMaxNp || (int64_t)(3 * p->nlev + 1) * p->K > kNoAllocMaxCnt) {
        std::fprintf(stderr,
                     "kore_solve_dev_noalloc: %lld padded unknowns in %d blocks exceed the fixed scratch "
                     "(%lld unknowns, %lld block counters); use kore_solve_dev\n",
                     (long long)p->np, p->K, (long long)kNoAllocMaxNp, (long long)kNoAllocMaxCnt);
        return KORE_EINVAL;
    }
    if (!p->factored) return KORE_ENOTFACTORED;
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
