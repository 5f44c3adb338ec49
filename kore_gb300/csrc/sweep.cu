// Block-tridiagonal sweeps, sparse products and the FP64 refinement loop.
//
// Solve of (A - sigma B) x = b with the factors of factor.cu (R = row scaling):
//     c   = s^-1 R b                      (s = ||b||_inf keeps complex64 in range)
//     z_i = S_i^-1 c_i                    all blocks in parallel
//     y_0 = z_0,      y_i = z_i - W_i y_{i-1}          forward, one block at a time
//     x_K-1 = y_K-1,  x_i = y_i - X_i x_{i+1}           backward
//     x  <- s x
// One cooperative persistent kernel runs the three phases with a bounded grid barrier
// between dependent blocks.  Each warp owns one row of the current block and
// prefetches that row of the next block's matrix into registers before it waits at
// the barrier, so the HBM stream of W_i / X_i overlaps the barrier latency.
//
// In mixed precision the factors are complex64 and the result is refined in FP64:
//     r = b - (A - sigma B) x,  x += M32^-1 r   until ||r||_inf <= tol (||M||_inf ||x||_inf + ||b||_inf).
#include "kore_internal.cuh"

namespace {

constexpr int kSweepThreads = 256;

template <typename C, int MAXT>
__device__ __forceinline__ void load_row(C (&rv)[MAXT], const C *__restrict__ row, int S, int lane) {
#pragma unroll
    for (int t = 0; t < MAXT; ++t) {
        const int j = lane + 32 * t;
        rv[t] = (j < S) ? __ldg(row + j) : czero<C>();
    }
}
__device__ __forceinline__ double2 ldcg(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2 *p) { return __ldcg(p); }
__device__ __forceinline__ void stcg(double2 *p, double2 v) { __stcg(p, v); }
__device__ __forceinline__ void stcg(float2 *p, float2 v) { __stcg(p, v); }

template <typename C, int MAXT>
__global__ void __launch_bounds__(kSweepThreads) k_sweep(
    int K, int S, const C *__restrict__ Sinv, const C *__restrict__ W, const C *__restrict__ X,
    const double2 *__restrict__ b, const double *__restrict__ rscale, const double *__restrict__ bnorm,
    C *__restrict__ z, C *__restrict__ y, double2 *__restrict__ out, int accumulate, unsigned *bar, int *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *vec = reinterpret_cast<C *>(smem_raw);
    GridBarrier gb;
    gb.init(bar, err);
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int gw = blockIdx.x * wpb + (threadIdx.x >> 5), nw = gridDim.x * wpb;
    const int64_t SS = (int64_t)S * S;
    const double bn = *bnorm;
    const double bscale = (bn > 0.0) ? 1.0 / bn : 1.0;
    const double oscale = (bn > 0.0) ? bn : 1.0;

    // phase 1: z = Sinv c, every row of every block
    for (int64_t row = gw; row < (int64_t)K * S; row += nw) {
        const int64_t i = row / S;
        const int k = (int)(row - i * S);
        const C *a = Sinv + i * SS + (int64_t)k * S;
        const double2 *bb = b + i * S;
        const double *rs = rscale + i * S;
        C acc = czero<C>();
        for (int j = lane; j < S; j += 32) acc = cfma(acc, __ldg(a + j), from_c128<C>((rs[j] * bscale) * bb[j]));
        acc = warp_sum(acc);
        if (lane == 0) stcg(z + row, acc);
    }
    const bool own = gw < S;
    C rv[MAXT];
    if (own) {
        stcg(y + gw, ldcg(z + gw));  // y_0 = z_0 (after the barrier everybody reads it)
        if (K > 1) load_row<C, MAXT>(rv, W + SS + (int64_t)gw * S, S, lane);
    }
    gb.sync();  // z complete, y_0 complete
    // phase 2: forward
    for (int i = 1; i < K; ++i) {
        for (int j = threadIdx.x; j < S; j += blockDim.x) vec[j] = ldcg(y + (int64_t)(i - 1) * S + j);
        __syncthreads();
        if (own) {
            C acc = czero<C>();
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int j = lane + 32 * t;
                if (j < S) acc = cfma(acc, rv[t], vec[j]);
            }
            acc = warp_sum(acc);
            if (lane == 0) stcg(y + (int64_t)i * S + gw, ldcg(z + (int64_t)i * S + gw) - acc);
            if (i + 1 < K) load_row<C, MAXT>(rv, W + (int64_t)(i + 1) * SS + (int64_t)gw * S, S, lane);
        }
        gb.sync();
    }
    // phase 3: backward (x overwrites y)
    if (own) {
        const int64_t idx = (int64_t)(K - 1) * S + gw;
        if (lane == 0) {
            const double2 v = oscale * to_c128(ldcg(y + idx));
            out[idx] = accumulate ? out[idx] + v : v;
        }
        if (K > 1) load_row<C, MAXT>(rv, X + (int64_t)(K - 2) * SS + (int64_t)gw * S, S, lane);
    }
    for (int i = K - 2; i >= 0; --i) {
        for (int j = threadIdx.x; j < S; j += blockDim.x) vec[j] = ldcg(y + (int64_t)(i + 1) * S + j);
        __syncthreads();
        if (own) {
            C acc = czero<C>();
#pragma unroll
            for (int t = 0; t < MAXT; ++t) {
                const int j = lane + 32 * t;
                if (j < S) acc = cfma(acc, rv[t], vec[j]);
            }
            acc = warp_sum(acc);
            if (lane == 0) {
                const int64_t idx = (int64_t)i * S + gw;
                const C xv = ldcg(y + idx) - acc;
                stcg(y + idx, xv);
                const double2 v = oscale * to_c128(xv);
                out[idx] = accumulate ? out[idx] + v : v;
            }
            if (i > 0) load_row<C, MAXT>(rv, X + (int64_t)(i - 1) * SS + (int64_t)gw * S, S, lane);
        }
        gb.sync();
    }
}

// max |v_p| over a padded vector -> red[blockIdx.x]
__global__ void k_absmax(int64_t np, const double2 *__restrict__ v, double *__restrict__ red) {
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
        if (threadIdx.x == 0) red[blockIdx.x] = t;
    }
}

// max of in[0..n) into *out (single CTA)
__global__ void k_reduce_max(const double *__restrict__ in, int n, double *__restrict__ out) {
    double mx = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, in[i]);
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) *out = t;
    }
}

// 8 lanes per row.  mode 0: y = B x.  mode 1: y = A x - lam B x.
// mode 2: y = b - (A x - lam B x) and per-CTA maxima of |y| and |x| into red.
constexpr int kRowLanes = 8;
__global__ void k_spmv(int64_t np, int mode, const int *__restrict__ arow, const int *__restrict__ acol,
                       const double2 *__restrict__ aval, const int *__restrict__ brow,
                       const int *__restrict__ bcol, const double *__restrict__ bval, int has_b, double lre,
                       double lim, const double2 *__restrict__ x, const double2 *__restrict__ rhs,
                       double2 *__restrict__ y, double *__restrict__ red) {
    const int sub = threadIdx.x & (kRowLanes - 1);
    const int64_t row0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kRowLanes;
    const int64_t rstride = ((int64_t)gridDim.x * blockDim.x) / kRowLanes;
    const double2 lam = mk(lre, lim);
    double rmax = 0.0, xmax = 0.0;
    for (int64_t p = row0; p < np + ((np % rstride) ? rstride - np % rstride : 0); p += rstride) {
        const bool live = p < np;
        double2 sa = mk(0.0, 0.0), sb = mk(0.0, 0.0);
        if (live) {
            if (mode != 0)
                for (int e = arow[p] + sub; e < arow[p + 1]; e += kRowLanes) sa = cfma(sa, aval[e], x[acol[e]]);
            if (has_b)
                for (int e = brow[p] + sub; e < brow[p + 1]; e += kRowLanes) sb = sb + bval[e] * x[bcol[e]];
        }
#pragma unroll
        for (int o = kRowLanes / 2; o > 0; o >>= 1) {
            sa.x += __shfl_down_sync(0xffffffffu, sa.x, o, kRowLanes);
            sa.y += __shfl_down_sync(0xffffffffu, sa.y, o, kRowLanes);
            sb.x += __shfl_down_sync(0xffffffffu, sb.x, o, kRowLanes);
            sb.y += __shfl_down_sync(0xffffffffu, sb.y, o, kRowLanes);
        }
        if (live && sub == 0) {
            double2 v;
            if (mode == 0) v = sb;
            else v = sa - lam * sb;
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
        __shared__ double sm[2][32];
        if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = rmax; sm[1][threadIdx.x >> 5] = xmax; }
        __syncthreads();
        if (threadIdx.x < 32) {
            const bool in = threadIdx.x < (blockDim.x >> 5);
            double a = in ? sm[0][threadIdx.x] : 0.0, c = in ? sm[1][threadIdx.x] : 0.0;
            a = warp_max_d(a);
            c = warp_max_d(c);
            if (threadIdx.x == 0) { red[2 * blockIdx.x] = a; red[2 * blockIdx.x + 1] = c; }
        }
    }
}

__global__ void k_gather(int64_t np, const int64_t *__restrict__ s2o, const double2 *__restrict__ orig,
                         double2 *__restrict__ padded) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = s2o[p];
        padded[p] = (o >= 0) ? orig[o] : mk(0.0, 0.0);
    }
}
__global__ void k_scatter(int64_t np, const int64_t *__restrict__ s2o, const double2 *__restrict__ padded,
                          double2 *__restrict__ orig) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = s2o[p];
        if (o >= 0) orig[o] = padded[p];
    }
}

template <typename C, int MAXT>
int launch_sweep_t(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate) {
    auto kern = k_sweep<C, MAXT>;
    const size_t smem = (size_t)p->S * sizeof(C);
    const C *Sinv = static_cast<const C *>(p->d_sinv);
    const C *W = static_cast<const C *>(p->d_W);
    const C *X = static_cast<const C *>(p->d_X);
    C *z = static_cast<C *>(p->d_zlo);
    C *y = static_cast<C *>(p->d_ylo);
    int K = p->K, S = p->S;
    KORE_CUDA_TRY(cudaMemsetAsync(p->d_bar, 0, sizeof(unsigned), p->stream));
    void *args[] = {&K, &S, (void *)&Sinv, (void *)&W, (void *)&X, (void *)&b, (void *)&p->d_rscale,
                    (void *)&bnorm, (void *)&z, (void *)&y, (void *)&x, &accumulate, (void *)&p->d_bar,
                    (void *)&p->d_err};
    dim3 grid(p->num_sms), block(kSweepThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kern, grid, block, args, smem, p->stream));
    KORE_LAUNCHED(1);
    return KORE_OK;
}

template <typename C>
int launch_sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate) {
    const int S = p->S;
    if (S <= 64) return launch_sweep_t<C, 2>(p, b, bnorm, x, accumulate);
    if (S <= 128) return launch_sweep_t<C, 4>(p, b, bnorm, x, accumulate);
    if (S <= 256) return launch_sweep_t<C, 8>(p, b, bnorm, x, accumulate);
    if (S <= 512) return launch_sweep_t<C, 16>(p, b, bnorm, x, accumulate);
    if (S <= 1024) return launch_sweep_t<C, 32>(p, b, bnorm, x, accumulate);
    return KORE_EINVAL;
}

int sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate) {
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, true));
    const int s = (p->prec == KORE_PREC_FP64) ? launch_sweep<double2>(p, b, bnorm, x, accumulate)
                                              : launch_sweep<float2>(p, b, bnorm, x, accumulate);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, false));
    return s;
}

// ||v||_inf of a padded vector into d_red[slot] (device)
int absmax(kore_plan *p, const double2 *v, int slot) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 1024u);
    k_absmax<<<grid, 256, 0, p->stream>>>(p->np, v, p->d_red + 2048);
    k_reduce_max<<<1, 1024, 0, p->stream>>>(p->d_red + 2048, (int)grid, p->d_red + slot);
    KORE_LAUNCHED(2);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

unsigned spmv_grid(kore_plan *p) {
    return std::min<unsigned>(kore_div_up(p->np * kRowLanes, 256), 1024u);
}

}  // namespace

int kore_spmv_b(kore_plan *p, const double2 *x, double2 *y) {
    if (!p->has_b) return KORE_EINVAL;
    k_spmv<<<spmv_grid(p), 256, 0, p->stream>>>(p->np, 0, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                 p->d_bval, 1, 0.0, 0.0, x, nullptr, y, nullptr);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_pencil(kore_plan *p, double lre, double lim, const double2 *x, double2 *y) {
    k_spmv<<<spmv_grid(p), 256, 0, p->stream>>>(p->np, 1, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                 p->d_bval, p->has_b ? 1 : 0, lre, lim, x, nullptr, y, nullptr);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_gather(kore_plan *p, const double2 *orig, double2 *padded) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_gather<<<grid, 256, 0, p->stream>>>(p->np, p->d_slot2orig, orig, padded);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_scatter(kore_plan *p, const double2 *padded, double2 *orig) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_scatter<<<grid, 256, 0, p->stream>>>(p->np, p->d_slot2orig, padded, orig);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

// d_red layout: [0, 2048) per-CTA partials of the residual kernel, [2048, 3072) partials
// of absmax, slots 4000.. scalars.
int kore_apply_inverse(kore_plan *p, const double2 *b, double2 *x, double tol, int *iters, double *resid) {
    if (!p->factored) return KORE_ENOTFACTORED;
    double *bn = p->d_red + 4000, *rn = p->d_red + 4001;
    KORE_TRY(absmax(p, b, 4000));
    KORE_TRY(sweep(p, b, bn, x, 0));
    int it = 0;
    double eta = -1.0;
    if (p->prec == KORE_PREC_MIXED) {
        if (!(tol > 0.0)) tol = 1e-14;
        double2 *r = p->d_v[5];
        const unsigned grid = spmv_grid(p);
        double prev = 1e300;
        for (it = 1; it <= 12; ++it) {
            k_spmv<<<grid, 256, 0, p->stream>>>(p->np, 2, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                p->d_bval, p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, x, b, r,
                                                p->d_red);
            KORE_LAUNCHED(1);
            KORE_CUDA_TRY(cudaMemcpyAsync(p->h_red, p->d_red, 2 * grid * sizeof(double), cudaMemcpyDeviceToHost,
                                          p->stream));
            KORE_CUDA_TRY(cudaMemcpyAsync(p->h_red + 4000, bn, sizeof(double), cudaMemcpyDeviceToHost, p->stream));
            KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
            KORE_TRY(kore_check_device_error(p));
            double rmax = 0.0, xmax = 0.0;
            for (unsigned c = 0; c < grid; ++c) {
                rmax = std::max(rmax, p->h_red[2 * c]);
                xmax = std::max(xmax, p->h_red[2 * c + 1]);
            }
            const double bmax = p->h_red[4000];
            const double den = p->minf * xmax + bmax;
            eta = (den > 0.0) ? rmax / den : 0.0;
            if (!(eta == eta)) return KORE_ENAN;
            // converged, or no longer improving (FP64 residual floor reached)
            if (eta <= tol || eta > 0.9 * prev) break;
            prev = eta;
            KORE_CUDA_TRY(cudaMemcpyAsync(rn, &rmax, sizeof(double), cudaMemcpyHostToDevice, p->stream));
            KORE_TRY(sweep(p, r, rn, x, 1));
        }
    }
    if (iters) *iters = it;
    if (resid) *resid = eta;
    return KORE_OK;
}
