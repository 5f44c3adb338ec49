// Shift-and-invert Krylov-Schur on the device.
//
// Restates what E.solve() does inside SLEPc for bin/solve.py:91-123 with
// `-st_type sinvert`: Krylov-Schur (Stewart 2001) on OP = (A - tau B)^-1 B.
//   * Arnoldi expansion with classical Gram-Schmidt in FP64 and SLEPc's default
//     refinement "if needed" (a second pass when the projection removed more than half
//     of ||w||^2, decided on the device);
//   * the projected matrix (ncv x ncv) is brought to complex Schur form on the device
//     (one CTA: Householder reduction to Hessenberg form, single-shift QR sweeps with
//     Wilkinson shifts and deflation, Givens reordering of the diagonal);
//   * the Schur form is ordered by SLEPc's comparison of the back-transformed values
//     lambda = tau + 1/theta (criterion `which`, target tau);
//   * Ritz estimates |b^T y_j| / ||y_j|| with the relative test  est_j / |theta_j| < tol;
//     the leading consecutive converged pairs count as converged (SLEPc's rule);
//   * thick restart keeping nconv + max(1, (ncv - nconv)/2) Schur vectors
//     (SLEPc's default keep = 0.5), at most maxit restarts;
//   * eigenvectors = Ritz vectors, purified by one more application of OP
//     (SLEPc's default for generalized problems under sinvert) and normalised to unit
//     2-norm (bin/solve.py:145-158).
// The basis size defaults to SLEPc's ncv = min(n, max(2 nev, nev + 15)) raised to 4 nev
// up to 64 (ncv_of below).
#include "kore_internal.cuh"
#include <cmath>
#include <algorithm>
#include <chrono>
#include <vector>

namespace {

constexpr int kMaxNcv = 64;
constexpr int kMaxTargets = 32;   // targets of one batched eigensolve (bits of a mask)

// ----------------------------------------------------------------------------- sort keys
// Ascending key = wanted first (the comparison functions of SLEPc's `which`) of an
// eigenvalue lambda = (lre, lim) for the target tau = (tre, tim).
__host__ __device__ inline double lambda_key(double2 lam, int which, double tre, double tim) {
    const double lre = lam.x, lim = lam.y;
    switch (which) {
        case KORE_WHICH_LM: return -hypot(lre, lim);
        case KORE_WHICH_SM: return hypot(lre, lim);
        case KORE_WHICH_LR: return -lre;
        case KORE_WHICH_SR: return lre;
        case KORE_WHICH_LI: return -lim;
        case KORE_WHICH_SI: return lim;
        case KORE_WHICH_TM: return hypot(lre - tre, lim - tim);
        case KORE_WHICH_TR: return fabs(lre - tre);
        case KORE_WHICH_TI: return fabs(lim - tim);
    }
    return 0.0;
}
// The same key for a Ritz value theta of OP = (A - sigma B)^-1 B: lambda = sigma + 1/theta,
// measured from the target tau.
__host__ __device__ inline double which_key(double2 theta, int which, double sre, double sim, double tre,
                                            double tim) {
    const double d = theta.x * theta.x + theta.y * theta.y;
    const double2 lam = (d > 0.0) ? mk(sre + theta.x / d, sim - theta.y / d) : mk(INFINITY, 0.0);
    return lambda_key(lam, which, tre, tim);
}

// Refinement tolerance that only the FP64 floor stops (the loop ends when the residual
// no longer decreases): used for the purifying application of the eigenvectors.
constexpr double kFloorRefineTol = 1e-300;
// Default relative residual of each OP application inside the Krylov iteration.
constexpr double kEigsRefineTol = 1e-16;

// ----------------------------------------------------------------------------- small Schur
struct SchurOut {
    double2 *T;       // m x m, column-major, upper triangular on exit
    double2 *Q;       // m x m, column-major
    double2 *Y;       // m x m, column j = unit eigenvector of T for T[j,j]
    double2 *theta;   // m
    double *est;      // m: relative Ritz estimates
    double2 *bnew;    // m: beta * Q[m-1, :]
    int *info;        // 0 ok, 1 QR failed to converge
};

__device__ inline double cabs_(double2 a) { return hypot(a.x, a.y); }

__device__ inline double2 csqrt_(double2 z) {
    const double r = hypot(z.x, z.y);
    if (r == 0.0) return mk(0.0, 0.0);
    double t = sqrt(0.5 * (r + fabs(z.x)));
    if (z.x >= 0.0) return mk(t, z.y / (2.0 * t));
    return mk(fabs(z.y) / (2.0 * t), copysign(t, z.y));
}

__device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }

__device__ __forceinline__ double2 shfl_xor_c(double2 v, int o) {
    v.x = __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y = __shfl_xor_sync(0xffffffffu, v.y, o);
    return v;
}

// G = [c s; -conj(s) c] with G [x; y] = [r; 0]; c = |x| / n, s = (x / |x|) conj(y) / n,
// n = sqrt(|x|^2 + |y|^2), evaluated with two reciprocal square roots.
__device__ __forceinline__ void givens_r(double2 x, double2 y, double &c, double2 &s) {
    const double a2 = abs2(x), b2 = abs2(y);
    if (b2 == 0.0) { c = 1.0; s = mk(0.0, 0.0); return; }
    if (a2 == 0.0) { c = 0.0; s = mk(1.0, 0.0); return; }
    const double rn = rsqrt(a2 + b2), ra = rsqrt(a2);
    c = a2 * ra * rn;
    s = (ra * rn) * (x * conjg(y));
}

// Apply G from the left to rows k, k+1 and G^H from the right to columns k, k+1 of H
// (rows [0, r1), columns [c0, m)), and G^H to columns k, k+1 of Q, in one parallel step.
// The FP64 dependency chain of a rotation is its latency (about 64 cycles per FP64
// operation on this GPU), so the 2 x 2 block where the row and column updates meet is
// split over lanes 0-3 of the last warp, one entry each, while the other warps update
// every other entry (one per thread): the two run on different SM sub-partitions.
__device__ __forceinline__ void apply_rot(double2 *H, double2 *Q, int m, int k, int c0, int r1, double c, double2 s) {
    const int tid = threadIdx.x, nt = blockDim.x - 32;
    if (tid >= nt) {
        if (tid >= nt + 4) return;
        const double2 h00 = H[k + k * m], h01 = H[k + (k + 1) * m], h10 = H[k + 1 + k * m],
                      h11 = H[k + 1 + (k + 1) * m];
        const int r = tid & 1, cc = (tid >> 1) & 1;   // output row k + r, column k + cc
        // rows of G [h]: row r of the rotated rows, at columns k and k+1
        const double2 ta = r ? c * h10 - conjg(s) * h00 : c * h00 + s * h10;   // column k
        const double2 tb = r ? c * h11 - conjg(s) * h01 : c * h01 + s * h11;   // column k+1
        const double2 out = cc ? c * tb - ta * s : c * ta + tb * conjg(s);
        __syncwarp(0xFu);
        H[k + r + (k + cc) * m] = out;
        return;
    }
    const int nrow = m - (k + 2);                     // columns k+2.. of rows k, k+1
    const int ncol = (r1 > k) ? k : r1;                // rows 0..k-1 of columns k, k+1
    const int nlow = (r1 > k + 2) ? 1 : 0;             // row k+2 of columns k, k+1
    const int nleft = (c0 < k) ? 1 : 0;                // column k-1 of rows k, k+1
    const int total = nrow + ncol + nlow + nleft + m;
    // Every item is a pair (a, b) of one matrix: rows k, k+1 of a column (G from the left,
    // u = s) or columns k, k+1 of a row (G^H from the right, u = conj(s)); both are
    // a' = c a + u b, b' = c b - conj(u) a.  Only the addressing differs between items,
    // so the FP64 arithmetic runs once per warp instead of once per divergent branch.
    for (int t = tid; t < total; t += nt) {
        int u = t, ia, step;
        bool left;
        double2 *M = H;
        if (u < nrow) {
            ia = k + (k + 2 + u) * m; step = 1; left = true;
        } else if ((u -= nrow) < ncol + nlow) {
            ia = ((u < ncol) ? u : k + 2) + k * m; step = m; left = false;
        } else if ((u -= ncol + nlow) < nleft) {
            ia = k + (k - 1) * m; step = 1; left = true;
        } else {
            u -= nleft;
            M = Q; ia = u + k * m; step = m; left = false;
        }
        const double2 a = M[ia], b = M[ia + step];
        const double2 us = left ? s : conjg(s);
        M[ia] = c * a + us * b;
        M[ia + step] = c * b - conjg(us) * a;
    }
}

// Per-target parameters of a batched k_schur launch: CTA t works on target t when bit t
// of `mask` is set; its Hbar, outputs T/Q/Y and theta/est/bnew lie at t times the strides.
struct SchurBatch {
    unsigned mask;
    int m[kMaxTargets], which[kMaxTargets];
    double tre[kMaxTargets], tim[kMaxTargets];   // targets
    double sre[kMaxTargets], sim[kMaxTargets];   // shifts of the slots' factors
    int64_t hstride, sqstride, vstride;
};

// One CTA of 128 threads per target (four warps, one per SM sub-partition, so the FP64
// updates of a rotation run on all four FP64 pipes).  Hbar: (m+1) x m column-major
// (ld m+1); row m is the residual row.
constexpr int kSchurT = 128;
__global__ void __launch_bounds__(kSchurT) k_schur(const double2 *__restrict__ Hbar0, const SchurBatch sb,
                                                   SchurOut out0) {
    const int tg = blockIdx.x;
    if (!((sb.mask >> tg) & 1u)) return;
    const int m = sb.m[tg], which = sb.which[tg];
    const double tre = sb.tre[tg], tim = sb.tim[tg], sre = sb.sre[tg], sim = sb.sim[tg];
    const double2 *Hbar = Hbar0 + tg * sb.hstride;
    const SchurOut out{out0.T + tg * sb.sqstride, out0.Q + tg * sb.sqstride, out0.Y + tg * sb.sqstride,
                       out0.theta + tg * sb.vstride, out0.est + tg * sb.vstride, out0.bnew + tg * sb.vstride,
                       out0.info + tg};
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *H = reinterpret_cast<double2 *>(smem_raw);  // m x m
    double2 *Q = H + m * m;                               // m x m
    double2 *Y = Q + m * m;                               // m x m
    __shared__ double2 vsh[kMaxNcv];
    __shared__ double key[kMaxNcv];
    __shared__ double red[4];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int ldh = m + 1;
    for (int idx = tid; idx < m * m; idx += kSchurT) {
        const int r = idx % m, c = idx / m;
        H[idx] = Hbar[r + c * ldh];
        Q[idx] = (r == c) ? mk(1.0, 0.0) : mk(0.0, 0.0);
    }
    __syncthreads();

    // --- Householder reduction to upper Hessenberg form
    for (int k = 0; k + 2 < m; ++k) {
        const int len = m - k - 1;
        double sq = 0.0;
        for (int i = tid; i < len; i += kSchurT) sq += abs2(H[k + 1 + i + k * m]);
        sq = warp_sum_d(sq);
        if (lane == 0) red[wid] = sq;
        __syncthreads();
        sq = red[0] + red[1] + red[2] + red[3];
        const double2 x0 = H[k + 1 + k * m];
        __syncthreads();
        if (!(sq - abs2(x0) > 0.0)) continue;
        const double xn = sqrt(sq);
        const double a0 = cabs_(x0);
        const double2 ph = (a0 > 0.0) ? mk(x0.x / a0, x0.y / a0) : mk(1.0, 0.0);
        // v = x + ph ||x|| e1, ||v||^2 = 2 ||x|| (||x|| + |x0|)
        const double vinv = rsqrt(2.0 * xn * (xn + a0));
        for (int i = tid; i < len; i += kSchurT) {
            double2 v = H[k + 1 + i + k * m];
            if (i == 0) v = v + xn * ph;
            vsh[i] = vinv * v;
        }
        __syncthreads();
        // H <- (I - 2 v v^H) H (rows k+1.., columns k..): four lanes per column, each
        // summing every fourth row, so the dependent FP64 chain is len / 4 long
        for (int base = 0; base < 4 * (m - k); base += kSchurT) {
            const int c = k + (base + tid) / 4, sub = tid & 3;
            const bool on = c < m;
            double2 t = mk(0.0, 0.0);
            if (on)
                for (int i = sub; i < len; i += 4) t = cfmaconj(t, vsh[i], H[k + 1 + i + c * m]);
            t = t + shfl_xor_c(t, 1);
            t = t + shfl_xor_c(t, 2);
            t = 2.0 * t;
            if (on)
                for (int i = sub; i < len; i += 4) H[k + 1 + i + c * m] = cfms(H[k + 1 + i + c * m], vsh[i], t);
        }
        __syncthreads();
        // H <- H (I - 2 v v^H), Q <- Q (I - 2 v v^H): two lanes per row
        for (int base = 0; base < 4 * m; base += kSchurT) {
            const int r = (base + tid) / 2, sub = tid & 1;
            const bool on = r < 2 * m;
            double2 *M = (r < m) ? H : Q;
            const int rr = (r < m) ? r : r - m;
            double2 t = mk(0.0, 0.0);
            if (on)
                for (int i = sub; i < len; i += 2) t = cfma(t, M[rr + (k + 1 + i) * m], vsh[i]);
            t = t + shfl_xor_c(t, 1);
            t = 2.0 * t;
            if (on)
                for (int i = sub; i < len; i += 2)
                    M[rr + (k + 1 + i) * m] = cfms(M[rr + (k + 1 + i) * m], t, conjg(vsh[i]));
        }
        __syncthreads();
        for (int i = 2 + tid; i < len + 1; i += kSchurT) H[k + i + k * m] = mk(0.0, 0.0);
        __syncthreads();
    }

    // --- shifted QR sweeps (complete Schur form, transformations accumulated in Q)
    const double eps = 2.220446049250313e-16;
    int hi = m - 1, iter = 0, total = 0, fail = 0;
    __shared__ int lred[kSchurT / 32];
    while (hi > 0) {
        // l = the largest index in [1, hi] whose subdiagonal entry is negligible, else 0:
        // one thread per candidate, maximum over the CTA
        int l = 0;
        for (int q = tid + 1; q <= hi; q += kSchurT) {
            double ref = cabs1(H[q - 1 + (q - 1) * m]) + cabs1(H[q + q * m]);
            if (ref == 0.0) ref = 1.0;
            if (cabs1(H[q + (q - 1) * m]) <= eps * ref) l = q;
        }
        l = __reduce_max_sync(0xffffffffu, l);
        if (lane == 0) lred[wid] = l;
        __syncthreads();
        for (int wv = 0; wv < kSchurT / 32; ++wv) l = max(l, lred[wv]);
        __syncthreads();
        if (l > 0 && tid == 0) H[l + (l - 1) * m] = mk(0.0, 0.0);
        __syncthreads();
        if (l == hi) { --hi; iter = 0; continue; }
        if (++total > 60 * m) { fail = 1; break; }
        ++iter;
        double2 mu;
        {
            const double2 a = H[hi - 1 + (hi - 1) * m], b = H[hi - 1 + hi * m];
            const double2 c = H[hi + (hi - 1) * m], d = H[hi + hi * m];
            if (iter % 10 == 0) {
                mu = d + mk(1.5 * fabs(c.x), 0.0);   // exceptional shift
            } else {
                const double2 half = 0.5 * (a - d);
                const double2 disc = csqrt_(half * half + b * c);
                const double2 m1 = 0.5 * (a + d) + disc, m2 = 0.5 * (a + d) - disc;
                mu = (abs2(m1 - d) < abs2(m2 - d)) ? m1 : m2;
            }
        }
        for (int k = l; k < hi; ++k) {
            double2 x, y;
            if (k == l) { x = H[l + l * m] - mu; y = H[l + 1 + l * m]; }
            else { x = H[k + (k - 1) * m]; y = H[k + 1 + (k - 1) * m]; }
            double c; double2 sn;
            givens_r(x, y, c, sn);
            __syncthreads();
            apply_rot(H, Q, m, k, (k > l) ? k - 1 : l, min(k + 3, hi + 1), c, sn);
            __syncthreads();
            if (k > l && tid == 0) H[k + 1 + (k - 1) * m] = mk(0.0, 0.0);
        }
        __syncthreads();
    }
    for (int idx = tid; idx < m * m; idx += kSchurT) {
        const int r = idx % m, c = idx / m;
        if (r > c) H[idx] = mk(0.0, 0.0);
    }
    __syncthreads();

    // --- order the diagonal by the `which` key: selection by adjacent swaps (Givens)
    for (int j = tid; j < m; j += kSchurT) key[j] = which_key(H[j + j * m], which, sre, sim, tre, tim);
    __syncthreads();
    for (int pos = 0; pos < m; ++pos) {
        int best = pos;
        double bk = key[pos];
        for (int j = pos + 1; j < m; ++j)
            if (key[j] < bk) { bk = key[j]; best = j; }
        for (int k = best - 1; k >= pos; --k) {
            const double2 t11 = H[k + k * m], t22 = H[k + 1 + (k + 1) * m], t12 = H[k + (k + 1) * m];
            double c; double2 sn;
            givens_r(t12, t22 - t11, c, sn);
            __syncthreads();
            apply_rot(H, Q, m, k, k, k + 2, c, sn);
            __syncthreads();
            if (tid == 0) {
                H[k + 1 + k * m] = mk(0.0, 0.0);
                const double t = key[k];
                key[k] = key[k + 1];
                key[k + 1] = t;
            }
            __syncthreads();
        }
    }

    // --- eigenvectors of T (one thread per eigenvalue), Ritz estimates
    const double beta = Hbar[m + (m - 1) * ldh].x;   // the only entry of the residual row
    for (int j = tid; j < m; j += kSchurT) {
        const double2 lam = H[j + j * m];
        double smin = eps * cabs1(lam);
        if (smin == 0.0) smin = 1e-300;
        for (int i = j + 1; i < m; ++i) Y[i + j * m] = mk(0.0, 0.0);
        Y[j + j * m] = mk(1.0, 0.0);
        for (int i = j - 1; i >= 0; --i) {
            double2 s = mk(0.0, 0.0);
            for (int l2 = i + 1; l2 <= j; ++l2) s = cfma(s, H[i + l2 * m], Y[l2 + j * m]);
            double2 den = H[i + i * m] - lam;
            if (cabs1(den) < smin) den = mk(smin, 0.0);
            const double dinv = 1.0 / abs2(den);
            Y[i + j * m] = -(dinv * (s * conjg(den)));
        }
        double yn = 0.0;
        for (int i = 0; i <= j; ++i) yn += abs2(Y[i + j * m]);
        const double yinv = rsqrt(yn);
        double2 bt = mk(0.0, 0.0);
        for (int i = 0; i <= j; ++i) {
            Y[i + j * m] = yinv * Y[i + j * m];
            bt = cfma(bt, Q[(m - 1) + i * m], Y[i + j * m]);
        }
        const double th = cabs_(lam);
        out.est[j] = (th > 0.0) ? beta * cabs_(bt) / th : INFINITY;
        out.theta[j] = lam;
        out.bnew[j] = beta * Q[(m - 1) + j * m];
    }
    __syncthreads();
    for (int idx = tid; idx < m * m; idx += kSchurT) {
        out.T[idx] = H[idx];
        out.Q[idx] = Q[idx];
        out.Y[idx] = Y[idx];
    }
    if (tid == 0) *out.info = fail;
}

// ----------------------------------------------------------------------------- tall-skinny kernels
// Every kernel below works on all targets of a batched eigensolve at once: grid.y (grid.x
// for the one-CTA kernels) is the target t, which takes part only when bit t of the
// launch's mask is set.  Per-target vectors are passed by value as arrays of device
// pointers, per-target column counts and indices in TCols.
struct TVec {
    double2 *p[kMaxTargets];
};
struct TCols {
    unsigned mask;
    int n[kMaxTargets];     // columns of V the launch uses (rows of G for k_gemm_vg)
    int j[kMaxTargets];     // column written (Hbar column; output columns for k_gemm_vg)
    int ld[kMaxTargets];    // leading dimension of the target's Hbar (ncv + 1), or of G
};
__device__ __forceinline__ bool in_mask(unsigned mask, int t) { return (mask >> t) & 1u; }

constexpr int kDotThreads = 256;
constexpr int kDotChunk = 8;
constexpr int kGridMax = 2048;                                        // CTAs of a tall-skinny kernel
constexpr int64_t kPartStride = (int64_t)kGridMax * (kMaxNcv + 1);   // per-target CTA partial sums
constexpr int64_t kHStride = 2 * (kMaxNcv + 1);                      // per-target [h1 | h2]
constexpr int64_t kHbarStride = (int64_t)(kMaxNcv + 1) * kMaxNcv;
constexpr int64_t kSqStride = (int64_t)kMaxNcv * kMaxNcv;
constexpr int64_t kVecStride = kMaxNcv + 1;

// Sums of 16 values over the 32 lanes of a warp with 16 FP64 additions per lane (a
// butterfly of 5 steps where each lane keeps half of its values and adds the partner's
// copy of that half) instead of the 80 of 16 separate warp sums; lanes 2k and 2k + 1
// return the total of value k.
__device__ __forceinline__ double warp_transpose_sum16(double (&v)[16], int lane) {
#pragma unroll
    for (int h = 8, m = 16; h >= 1; h >>= 1, m >>= 1) {
        const bool up = lane & m;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const double send = up ? v[i] : v[i + h];
            const double keep = up ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, m);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// Target t: partial_t[b*nc + c] = sum over the CTA's rows of conj(V_t[:,c]) w_t for
// c < ncol_t and, with with_norm, entry c = ncol_t = sum |w_t|^2 (nc = ncol_t + with_norm).
// run (may be null): target t returns at once unless run[t] != 0.
__global__ void __launch_bounds__(kDotThreads) k_mdot(int64_t np, TVec V, TVec w, double2 *__restrict__ partial0,
                                                      int with_norm, const int *__restrict__ run, TCols tc) {
    const int tg = blockIdx.y;
    if (!in_mask(tc.mask, tg) || (run && run[tg] == 0)) return;
    const double2 *__restrict__ Vt = V.p[tg];
    const double2 *__restrict__ wt = w.p[tg];
    double2 *__restrict__ partial = partial0 + tg * kPartStride;
    __shared__ double sm[kDotThreads / 32][2 * kDotChunk];
    const int ncol = tc.n[tg];
    const int nc = ncol + with_norm;
    for (int c0 = 0; c0 < nc; c0 += kDotChunk) {
        double2 acc[kDotChunk];
#pragma unroll
        for (int t = 0; t < kDotChunk; ++t) acc[t] = mk(0.0, 0.0);
        // two rows per step, both rows' loads issued before their products: the CTA's
        // warps meet at every chunk's reduction, so a row's load latency is not hidden by
        // other warps' products
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        for (; r + stride < np; r += 2 * stride) {
            const int64_t r2 = r + stride;
            const double2 wa = wt[r], wb = wt[r2];
            double2 va[kDotChunk], vb[kDotChunk];
#pragma unroll
            for (int t = 0; t < kDotChunk; ++t) {
                const bool col = c0 + t < ncol;
                va[t] = col ? Vt[r + (int64_t)(c0 + t) * np] : wa;
                vb[t] = col ? Vt[r2 + (int64_t)(c0 + t) * np] : wb;
            }
#pragma unroll
            for (int t = 0; t < kDotChunk; ++t)
                if (c0 + t < nc) acc[t] = cfmaconj(cfmaconj(acc[t], va[t], wa), vb[t], wb);
        }
        if (r < np) {
            const double2 wr = wt[r];
#pragma unroll
            for (int t = 0; t < kDotChunk; ++t)
                if (c0 + t < nc) acc[t] = cfmaconj(acc[t], (c0 + t < ncol) ? Vt[r + (int64_t)(c0 + t) * np] : wr, wr);
        }
        // warp sums of the 2 kDotChunk doubles: even lane L ends with value L / 2
        double v[2 * kDotChunk];
#pragma unroll
        for (int t = 0; t < kDotChunk; ++t) { v[2 * t] = acc[t].x; v[2 * t + 1] = acc[t].y; }
        const int lane = threadIdx.x & 31;
        const double tot = warp_transpose_sum16(v, lane);
        if ((lane & 1) == 0) sm[threadIdx.x >> 5][lane >> 1] = tot;
        __syncthreads();
        if (threadIdx.x < kDotChunk && c0 + (int)threadIdx.x < nc) {
            double2 s = mk(0.0, 0.0);
            for (int wv = 0; wv < kDotThreads / 32; ++wv)
                s = s + mk(sm[wv][2 * threadIdx.x], sm[wv][2 * threadIdx.x + 1]);
            partial[blockIdx.x * (int64_t)nc + c0 + threadIdx.x] = s;
        }
        __syncthreads();
    }
}

// Target t (grid.y), column c (grid.x): h_t[c] (+)= sum_b partial_t[b*nc + c] with
// nc = ncol_t + with_norm; returns at once unless run[t] != 0 (when run is given).
__global__ void k_mdot_reduce(int nblk, const double2 *__restrict__ partial0, int64_t pstride,
                              double2 *__restrict__ h0, int accumulate, const int *__restrict__ run, TCols tc,
                              int with_norm) {
    const int tg = blockIdx.y;
    if (!in_mask(tc.mask, tg) || (run && run[tg] == 0)) return;
    const int nc = tc.n[tg] + with_norm;
    const int c = blockIdx.x;
    if (c >= nc) return;
    const double2 *__restrict__ partial = partial0 + tg * pstride;
    double2 *__restrict__ h = h0 + tg * kHStride;
    double2 s = mk(0.0, 0.0);
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) s = s + partial[(int64_t)b * nc + c];
    s = warp_sum(s);
    __shared__ double2 sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = mk(0.0, 0.0);
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t = t + sm[wv];
        h[c] = accumulate ? h[c] + t : t;
    }
}

// w_t -= V_t h_t (ncol_t columns); returns at once unless run[t] != 0 (when run is given)
__global__ void k_mgs_update(int64_t np, TVec V, const double2 *__restrict__ h0, TVec w,
                             const int *__restrict__ run, TCols tc) {
    const int tg = blockIdx.y;
    if (!in_mask(tc.mask, tg) || (run && run[tg] == 0)) return;
    const double2 *__restrict__ Vt = V.p[tg];
    double2 *__restrict__ wt = w.p[tg];
    const int ncol = tc.n[tg];
    __shared__ double2 hs[kMaxNcv + 1];
    for (int c = threadIdx.x; c < ncol; c += blockDim.x) hs[c] = h0[tg * kHStride + c];
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
        double2 acc = wt[r];
        for (int c = 0; c < ncol; ++c) acc = cfms(acc, Vt[r + (int64_t)c * np], hs[c]);
        wt[r] = acc;
    }
}

// partial_t[b] = sum of |w_t|^2 over CTA b's rows (grid.y = target)
__global__ void k_nrm2_partial(int64_t np, TVec w, double *__restrict__ partial0, unsigned mask) {
    const int tg = blockIdx.y;
    if (!in_mask(mask, tg)) return;
    const double2 *__restrict__ wt = w.p[tg];
    double s = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x)
        s += abs2(wt[r]);
    s = warp_sum_d(s);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t += sm[wv];
        partial0[tg * (int64_t)kGridMax + blockIdx.x] = t;
    }
}

// Refinement decision of classical Gram-Schmidt (SLEPc's default, refinement "if needed"
// with eta = 1/sqrt(2)), one CTA per target: h1[ncol].x = ||w||^2 before the first pass;
// the norm after it is sqrt(||w||^2 - sum |h1_c|^2) (exact for orthonormal V); a second
// pass runs when that is below eta ||w||.  Clears h2, which a skipped second pass leaves
// untouched.
__global__ void k_refine_decide(double2 *__restrict__ h0, int *__restrict__ run2, TCols tc) {
    const int tg = blockIdx.x;
    if (!in_mask(tc.mask, tg)) return;
    const double2 *__restrict__ h1 = h0 + tg * kHStride;
    double2 *__restrict__ h2 = h0 + tg * kHStride + (kMaxNcv + 1);
    const int ncol = tc.n[tg];
    __shared__ double sm[32];
    double s = 0.0;
    for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
        s += abs2(h1[c]);
        h2[c] = mk(0.0, 0.0);
    }
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t += sm[wv];
        const double onrm2 = h1[ncol].x;
        run2[tg] = (onrm2 - t < 0.5 * onrm2) ? 1 : 0;
    }
}

// One CTA per target: beta_t = sqrt(sum of its partials); with set_col, Hbar_t[j+1, j] =
// beta_t and h_t (ncol_t entries) becomes column j of Hbar_t (j = tc.j[t], ld tc.ld[t]).
__global__ void k_finish_col(int nblk, const double *__restrict__ partial0, const double2 *__restrict__ h0,
                             double2 *__restrict__ Hbar0, double *__restrict__ beta0, TCols tc, int set_col) {
    const int tg = blockIdx.x;
    if (!in_mask(tc.mask, tg)) return;
    const double *__restrict__ partial = partial0 + tg * (int64_t)kGridMax;
    __shared__ double sm[32];
    double s = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += partial[b];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    double2 *__restrict__ Hbar = Hbar0 + tg * kHbarStride;
    const int j = tc.j[tg], ld = tc.ld[tg];
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t += sm[wv];
        const double beta = sqrt(t);
        beta0[tg] = beta;
        if (set_col) Hbar[(j + 1) + (int64_t)j * ld] = mk(beta, 0.0);
    }
    if (set_col)
        for (int c = threadIdx.x; c < tc.n[tg]; c += blockDim.x) Hbar[c + (int64_t)j * ld] = h0[tg * kHStride + c];
}

// dst_t = src_t / beta_t (beta_t > 0), else 0; src and dst may be the same vector
__global__ void k_scale_copy(int64_t np, TVec src, const double *__restrict__ beta0, TVec dst, unsigned mask) {
    const int tg = blockIdx.y;
    if (!in_mask(mask, tg)) return;
    const double s = beta0[tg];
    const double inv = (s > 0.0) ? 1.0 / s : 0.0;
    const double2 *__restrict__ a = src.p[tg];
    double2 *__restrict__ b = dst.p[tg];
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x)
        b[r] = inv * a[r];
}

// dst_t = src_t (np entries)
// out = sum of the n columns of V (column k at V + k * np)
__global__ void k_sum_cols(int64_t np, const double2 *__restrict__ V, int n, double2 *__restrict__ out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
        double2 s = mk(0.0, 0.0);
        for (int k = 0; k < n; ++k) s = s + V[(int64_t)k * np + r];
        out[r] = s;
    }
}

// v <- v / ||v||_2 (one CTA; a zero vector is left as it is)
__global__ void k_unit(int64_t np, double2 *__restrict__ v) {
    double s = 0.0;
    for (int64_t r = threadIdx.x; r < np; r += blockDim.x) s += abs2(v[r]);
    s = warp_sum_d(s);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sm[q];
    if (!(t > 0.0)) return;
    const double inv = rsqrt(t);
    for (int64_t r = threadIdx.x; r < np; r += blockDim.x) v[r] = inv * v[r];
}

// y <- y + x
__global__ void k_add(int64_t np, const double2 *__restrict__ x, double2 *__restrict__ y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x)
        y[r] = y[r] + x[r];
}

__global__ void k_copy_vecs(int64_t np, TVec src, TVec dst, unsigned mask) {
    const int tg = blockIdx.y;
    if (!in_mask(mask, tg)) return;
    const double2 *__restrict__ a = src.p[tg];
    double2 *__restrict__ b = dst.p[tg];
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x)
        b[r] = a[r];
}

// Target t: Vout_t[:, c] = V_t[:, 0:m_t] G_t[:, c] for c < ncol_t, with m_t = tc.n[t],
// ncol_t = tc.j[t] and G_t column-major with leading dimension tc.ld[t].
constexpr int kGemmChunk = 8;
__global__ void k_gemm_vg(int64_t np, TVec V, TVec G, TVec Vout, TCols tc) {
    const int tg = blockIdx.y;
    if (!in_mask(tc.mask, tg)) return;
    const int m = tc.n[tg], ncol = tc.j[tg], ldg = tc.ld[tg];
    const double2 *__restrict__ Vt = V.p[tg];
    const double2 *__restrict__ Gt = G.p[tg];
    double2 *__restrict__ Vo = Vout.p[tg];
    __shared__ double2 gs[kMaxNcv * kGemmChunk];
    for (int c0 = 0; c0 < ncol; c0 += kGemmChunk) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < m * kGemmChunk; idx += blockDim.x) {
            const int j = idx % m, t = idx / m;
            gs[j * kGemmChunk + t] = (c0 + t < ncol) ? Gt[j + (int64_t)(c0 + t) * ldg] : mk(0.0, 0.0);
        }
        __syncthreads();
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
            double2 acc[kGemmChunk];
#pragma unroll
            for (int t = 0; t < kGemmChunk; ++t) acc[t] = mk(0.0, 0.0);
            for (int j = 0; j < m; ++j) {
                const double2 v = Vt[r + (int64_t)j * np];
#pragma unroll
                for (int t = 0; t < kGemmChunk; ++t) acc[t] = cfma(acc[t], v, gs[j * kGemmChunk + t]);
            }
#pragma unroll
            for (int t = 0; t < kGemmChunk; ++t)
                if (c0 + t < ncol) Vo[r + (int64_t)(c0 + t) * np] = acc[t];
        }
    }
}

// One CTA per target: Hbar_t <- [T_t[0:p,0:p]; bnew_t[0:p]] (ld m+1), other entries zero,
// with m = tc.ld[t] - 1 and p = tc.n[t] (the kept Schur vectors)
__global__ void k_restart_h(const double2 *__restrict__ T0, const double2 *__restrict__ bnew0,
                            double2 *__restrict__ Hbar0, TCols tc) {
    const int tg = blockIdx.x;
    if (!in_mask(tc.mask, tg)) return;
    const int ld = tc.ld[tg], m = ld - 1, p = tc.n[tg];
    const double2 *__restrict__ T = T0 + tg * kSqStride;
    const double2 *__restrict__ bnew = bnew0 + tg * kVecStride;
    double2 *__restrict__ Hbar = Hbar0 + tg * kHbarStride;
    for (int idx = threadIdx.x; idx < ld * m; idx += blockDim.x) {
        const int r = idx % ld, c = idx / ld;
        double2 v = mk(0.0, 0.0);
        if (c < p) {
            if (r < p) v = T[r + c * m];
            else if (r == p) v = bnew[c];
        }
        Hbar[idx] = v;
    }
}

// Least-squares Rayleigh quotient of an approximate eigenvector x of A x = lambda B x:
// lambda = (B x)^H (A x) / ||B x||^2 minimises ||A x - lambda B x||_2 over lambda.
// Target t: partial_t[2 b] = sum conj(bx) ax, partial_t[2 b + 1].x = sum |bx|^2 over
// CTA b's rows.
__global__ void k_rq_partial(int64_t np, TVec ax, TVec bx, double2 *__restrict__ partial0, unsigned mask) {
    const int tg = blockIdx.y;
    if (!in_mask(mask, tg)) return;
    const double2 *__restrict__ a = ax.p[tg];
    const double2 *__restrict__ bv = bx.p[tg];
    double2 num = mk(0.0, 0.0);
    double den = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
        const double2 b = bv[r];
        num = cfmaconj(num, b, a[r]);
        den += abs2(b);
    }
    num = warp_sum(num);
    den = warp_sum_d(den);
    __shared__ double2 sn[32];
    __shared__ double sd[32];
    if ((threadIdx.x & 31) == 0) { sn[threadIdx.x >> 5] = num; sd[threadIdx.x >> 5] = den; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { num = num + sn[w]; den += sd[w]; }
        double2 *partial = partial0 + tg * kPartStride;
        partial[2 * blockIdx.x] = num;
        partial[2 * blockIdx.x + 1] = mk(den, 0.0);
    }
}
// One CTA per target: lam_t[k] = sum of numerators / sum of denominators (fixed order)
__global__ void k_rq_finish(int nblk, const double2 *__restrict__ partial0, double2 *__restrict__ lam0, int k,
                            unsigned mask) {
    const int tg = blockIdx.x;
    if (!in_mask(mask, tg)) return;
    const double2 *__restrict__ partial = partial0 + tg * kPartStride;
    double2 num = mk(0.0, 0.0);
    double den = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) { num = num + partial[2 * b]; den += partial[2 * b + 1].x; }
    num = warp_sum(num);
    den = warp_sum_d(den);
    __shared__ double2 sn[32];
    __shared__ double sd[32];
    if ((threadIdx.x & 31) == 0) { sn[threadIdx.x >> 5] = num; sd[threadIdx.x >> 5] = den; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { num = num + sn[w]; den += sd[w]; }
        lam0[tg * kVecStride + k] = (den > 0.0) ? mk(num.x / den, num.y / den) : mk(NAN, NAN);
    }
}

// Clear the refinement statistics of shift s for a new target (the sweep counters,
// which count launches for the whole plan, are kept).
__global__ void k_ir_slot_reset(IrState *st, int s) {
    IrState &x = st[s];
    x.done = 0; x.nan = 0; x.iters = 0; x.iters_cur = 0; x.iters_max = 0; x.applies = 0;
    x.prev = 0.0; x.eta_max = 0.0;
}

// ----------------------------------------------------------------------------- host helpers
// Device workspace of a batched eigensolve; every per-target array lies at t times its
// stride.  w, t1 and xin are T x np (target t at t * np).
struct Ctx {
    kore_plan *p;
    int T;
    int64_t np;
    unsigned grid;
    double2 *w, *t1, *xin;
    double2 *Hbar, *Tm, *Q, *Y, *theta, *bnew, *lam, *h, *partial;
    double *est, *dpart, *beta;
    int *info, *run2;
    double refine_tol;
    std::vector<int> applies;   // applications of OP per target
};

// bytes of the small per-target arrays (double2 units) of T targets
size_t small_elems(int T) {
    const size_t t = (size_t)T;
    return t * (kHbarStride + 3 * kSqStride + 3 * kVecStride + kHStride + kPartStride) +
           (t * (kVecStride + kGridMax + 8) + 1) / 2 + (2 * t + 3) / 4 + 4;
}

void carve_small(Ctx &c, double2 *base) {
    const int64_t T = c.T;
    c.Hbar = base;
    c.Tm = c.Hbar + T * kHbarStride;
    c.Q = c.Tm + T * kSqStride;
    c.Y = c.Q + T * kSqStride;
    c.theta = c.Y + T * kSqStride;
    c.bnew = c.theta + T * kVecStride;
    c.lam = c.bnew + T * kVecStride;
    c.h = c.lam + T * kVecStride;
    c.partial = c.h + T * kHStride;
    c.est = reinterpret_cast<double *>(c.partial + T * kPartStride);
    c.dpart = c.est + T * kVecStride;
    c.beta = c.dpart + T * kGridMax;
    c.info = reinterpret_cast<int *>(c.beta + T * 8);
    c.run2 = c.info + T;
}

// Deterministic complex standard normal start vector (SplitMix64 + Box-Muller).
static uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static void start_vector(int64_t n, uint64_t seed, double2 *v) {
    uint64_t s = seed;
    const double two_pi = 6.283185307179586476925286766559;
    for (int64_t i = 0; i < n; ++i) {
        double u1 = ((splitmix(s) >> 11) + 1) * (1.0 / 9007199254740993.0);
        double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
        double r = std::sqrt(-2.0 * std::log(u1));
        v[i] = mk(r * std::cos(two_pi * u2), r * std::sin(two_pi * u2));
    }
}

TVec contiguous(double2 *base, int T, int64_t np) {
    TVec v;
    for (int t = 0; t < kMaxTargets; ++t) v.p[t] = (t < T) ? base + t * np : nullptr;
    return v;
}

// w_t = OP v_t = (A - tau_t B)^-1 B v_t for the targets in mask (one multi-shift sparse
// product and one multi-shift solve; the other targets' w is left as it is)
int apply_op(Ctx &c, const TVec &v, unsigned mask, const double *shift_tols = nullptr) {
    kore_plan *p = c.p;
    const double2 *x = v.p[0];
    if (c.T > 1) {
        k_copy_vecs<<<dim3(c.grid, c.T), 256, 0, p->stream>>>(c.np, v, contiguous(c.xin, c.T, c.np), mask);
        KORE_LAUNCHED(1);
        x = c.xin;
    }
    KORE_TRY(kore_spmv_b_shifts(p, x, c.t1, mask));
    for (int t = 0; t < c.T; ++t)
        if ((mask >> t) & 1u) c.applies[t] += 1;
    return kore_apply_inverse(p, c.t1, c.w, c.refine_tol, mask, shift_tols);
}

// For each target t in tc.mask: orthogonalise w_t against V_t[:, 0:ncol_t] (classical
// Gram-Schmidt with refinement if needed), write h and beta into column j_t of Hbar_t and
// set V_t[:, j_t + 1] = w_t / beta.
int orthonormalise(Ctx &c, const TVec &V, const TCols &tc) {
    kore_plan *p = c.p;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 3, true));
    int nmax = 0;
    for (int t = 0; t < c.T; ++t)
        if ((tc.mask >> t) & 1u) nmax = std::max(nmax, tc.n[t]);
    const TVec w = contiguous(c.w, c.T, c.np);
    double2 *h1 = c.h, *h2 = c.h + (kMaxNcv + 1);
    const dim3 g2(c.grid, c.T);
    // first pass, with ||w||^2 as entry ncol of h1
    k_mdot<<<g2, kDotThreads, 0, p->stream>>>(c.np, V, w, c.partial, 1, nullptr, tc);
    k_mdot_reduce<<<dim3(nmax + 1, c.T), 256, 0, p->stream>>>((int)c.grid, c.partial, kPartStride, h1, 0, nullptr,
                                                               tc, 1);
    k_mgs_update<<<g2, 256, 0, p->stream>>>(c.np, V, h1, w, nullptr, tc);
    k_refine_decide<<<c.T, 256, 0, p->stream>>>(c.h, c.run2, tc);
    // second pass if needed
    k_mdot<<<g2, kDotThreads, 0, p->stream>>>(c.np, V, w, c.partial, 0, c.run2, tc);
    k_mdot_reduce<<<dim3(nmax, c.T), 256, 0, p->stream>>>((int)c.grid, c.partial, kPartStride, h2, 0, c.run2, tc, 0);
    k_mgs_update<<<g2, 256, 0, p->stream>>>(c.np, V, h2, w, c.run2, tc);
    KORE_LAUNCHED(7);
    // h = h1 + h2
    k_mdot_reduce<<<dim3(nmax, c.T), 32, 0, p->stream>>>(1, h2, kHStride, h1, 1, nullptr, tc, 0);
    k_nrm2_partial<<<g2, 256, 0, p->stream>>>(c.np, w, c.dpart, tc.mask);
    k_finish_col<<<c.T, 256, 0, p->stream>>>((int)c.grid, c.dpart, c.h, c.Hbar, c.beta, tc, 1);
    TVec vnext;
    for (int t = 0; t < kMaxTargets; ++t)
        vnext.p[t] = (t < c.T && ((tc.mask >> t) & 1u)) ? V.p[t] + (int64_t)(tc.j[t] + 1) * c.np : nullptr;
    k_scale_copy<<<g2, 256, 0, p->stream>>>(c.np, w, c.beta, vnext, tc.mask);
    KORE_LAUNCHED(4);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 3, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

// One slot of the batched eigensolve engine: the target it serves and where that
// target's Krylov-Schur stands.
struct Slot {
    bool busy = false;
    EigsTarget tgt;
    int phase = 2;         // 0 expanding the basis, 1 purifying the eigenvectors, 2 idle
    int m = 0, nev = 0;    // ncv, nev
    int j = 0;             // basis vectors formed: the next step writes column j + 1
    int restarts = 0, nconv = 0, applies = 0;
    double2 *V = nullptr, *Vt = nullptr;   // basis and restart buffers (swapped at restarts)
    std::vector<double2> theta;            // Ritz values of the last Schur form
    int nout = 0, k = 0, pstep = 0;        // purification: vectors, next vector, applications done on it
    bool valid = false;                    // the slot's factors are those of p->sigmas[s]
};

// The state of one engine run.
struct Run {
    kore_plan *p;
    Ctx c;
    int T;                    // slots (= the plan's shifts)
    int M;                    // largest ncv a slot's buffers hold
    EigsSource *src;
    std::vector<Slot> sl;
    SchurBatch sb{};
    std::chrono::steady_clock::time_point t0;
};

// Default basis size: SLEPc's max(2 nev, nev + 15), raised to 4 nev up to the largest
// basis the projected-problem kernel holds.  An operator application (a sweep and its
// refinement, milliseconds at full size) costs far more than the orthogonalisation and
// the projected problem of a larger basis, and the larger basis needs fewer restarts and
// fewer applications: on the 240k-unknown shell at nev = 16, 64 vectors take 191
// applications and 5 restarts against 303-350 and 22-26 with 32.
// The shift of the spectral transformation: the target unless set apart (SLEPc -st_shift).
inline double2 shift_of(const kore_eps_opts &o) {
    return o.has_shift ? mk(o.shift_re, o.shift_im) : mk(o.target_re, o.target_im);
}

int ncv_of(const kore_plan *p, const kore_eps_opts &o) {
    if (o.ncv > 0) return o.ncv;
    const int m = std::max(std::max(2 * o.nev, o.nev + 15), std::min(kMaxNcv, 4 * o.nev));
    return (int)std::min<int64_t>(p->n, m);
}

// KORE_OK when the options can run in a slot of this engine
int check_opts(const kore_plan *p, const kore_eps_opts &o, int M) {
    if (o.nev <= 0 || o.purify < 0 || !(o.reuse_radius >= 0.0)) return KORE_EINVAL;
    if (o.has_shift && !(std::isfinite(o.shift_re) && std::isfinite(o.shift_im))) return KORE_EINVAL;
    // shift-and-invert needs a target criterion: SLEPc's EPSSetUp refuses the others
    // under -st_type sinvert, the only spectral transformation of the kore path
    if (o.which != KORE_WHICH_TM && o.which != KORE_WHICH_TR && o.which != KORE_WHICH_TI) return KORE_EINVAL;
    const int m = ncv_of(p, o);
    if (m > kMaxNcv || m <= o.nev || m > p->n || m > M) return KORE_EINVAL;
    return KORE_OK;
}

// Start target t in the free slot s: factorise its shift there unless the slot already
// holds it, and give the basis its normalised start vector.
int start_target(Run &r, int s, const EigsTarget &t) {
    kore_plan *p = r.p;
    Ctx &c = r.c;
    const kore_eps_opts &ot = t.opts;
    Slot &x = r.sl[s];
    const double2 sh = shift_of(ot);
    const bool reuse = x.valid && p->sigmas[s].x == sh.x && p->sigmas[s].y == sh.y;
    if (!reuse) {
        x.valid = false;
        KORE_TRY(kore_factor_slot(p, s, sh.x, sh.y));
        x.valid = true;
    }
    x.busy = true;
    x.tgt = t;
    x.tgt.reused = reuse ? 1 : 0;
    x.phase = 0;
    x.m = ncv_of(p, ot);
    x.nev = ot.nev;
    x.j = 0; x.restarts = 0; x.nconv = 0; x.applies = 0;
    x.nout = 0; x.k = 0; x.pstep = 0;
    r.sb.m[s] = x.m; r.sb.which[s] = ot.which; r.sb.tre[s] = ot.target_re; r.sb.tim[s] = ot.target_im;
    r.sb.sre[s] = sh.x; r.sb.sim[s] = sh.y;
    // start vector: seeded (original order) -> padded; warm: the seeded vector and the
    // slot's warm vector, both of unit norm, added.  The warm vector alone would not do:
    // it lies in the invariant subspace of the previous target's eigenvectors, where the
    // Krylov space would stop, so the seeded part keeps the other directions in it.
    // Then normalised into column 0.
    double2 *orig = c.xin + (int64_t)s * c.np, *pad = c.w + (int64_t)s * c.np;
    std::vector<double2> hv((size_t)p->n);
    start_vector(p->n, ot.seed, hv.data());
    const bool warm = ot.warm && s < (int)p->warm_ok.size() && p->warm_ok[s];
    if (warm) {
        double nn = 0.0;
        for (const double2 &e : hv) nn += e.x * e.x + e.y * e.y;
        const double inv = nn > 0.0 ? 1.0 / std::sqrt(nn) : 1.0;
        for (double2 &e : hv) { e.x *= inv; e.y *= inv; }
    }
    KORE_CUDA_TRY(cudaMemcpyAsync(orig, hv.data(), hv.size() * sizeof(double2), cudaMemcpyHostToDevice, p->stream));
    KORE_TRY(kore_gather(p, orig, pad));
    if (warm) {
        k_add<<<c.grid, 256, 0, p->stream>>>(c.np, p->d_warm + (int64_t)s * c.np, pad);
        KORE_LAUNCHED(1);
        x.tgt.warm_started = 1;
    }
    TCols tc{};
    tc.mask = 1u << s;
    tc.n[s] = 0; tc.j[s] = -1; tc.ld[s] = x.m + 1;
    TVec src, dst;
    for (int u = 0; u < kMaxTargets; ++u) src.p[u] = dst.p[u] = nullptr;
    src.p[s] = pad; dst.p[s] = x.V;
    k_nrm2_partial<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(c.np, src, c.dpart, tc.mask);
    k_finish_col<<<r.T, 256, 0, p->stream>>>((int)c.grid, c.dpart, c.h, c.Hbar, c.beta, tc, 0);
    k_scale_copy<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(c.np, src, c.beta, dst, tc.mask);
    k_ir_slot_reset<<<1, 1, 0, p->stream>>>(p->d_ir, s);
    KORE_LAUNCHED(4);
    KORE_CUDA_TRY(cudaMemsetAsync(c.Hbar + s * kHbarStride, 0, sizeof(double2) * kHbarStride, p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));   // hv is released on return
    return KORE_OK;
}

// Fill the free slots from the source; a target whose options or start fail is handed
// back at once with that status.  Slots that hold a target's shift are preferred.
int fill_slots(Run &r) {
    for (;;) {
        int nfree = 0;
        for (int s = 0; s < r.T; ++s) nfree += !r.sl[s].busy;
        if (nfree == 0) return KORE_OK;
        EigsTarget t;
        if (!r.src->next(&t)) return KORE_OK;
        const int rc = check_opts(r.p, t.opts, r.M);
        if (rc != KORE_OK) {
            r.src->finished(t, rc);
            continue;
        }
        int s = -1;
        const double2 sh = shift_of(t.opts);
        for (int u = 0; u < r.T && s < 0; ++u)
            if (!r.sl[u].busy && r.sl[u].valid && r.p->sigmas[u].x == sh.x && r.p->sigmas[u].y == sh.y) s = u;
        if (s < 0 && t.opts.reuse_radius > 0.0 && !t.opts.has_shift) {
            // the idle slot whose factors lie nearest the target, within the radius: run
            // there with that slot's shift (started warm only if the target asks for it)
            double best = t.opts.reuse_radius;
            for (int u = 0; u < r.T; ++u)
                if (!r.sl[u].busy && r.sl[u].valid) {
                    const double d = hypot(r.p->sigmas[u].x - t.opts.target_re, r.p->sigmas[u].y - t.opts.target_im);
                    if (d <= best) { best = d; s = u; }
                }
            if (s >= 0) {
                t.opts.has_shift = 1;
                t.opts.shift_re = r.p->sigmas[s].x;
                t.opts.shift_im = r.p->sigmas[s].y;
            }
        }
        for (int u = 0; u < r.T && s < 0; ++u)
            if (!r.sl[u].busy) s = u;
        const int st = start_target(r, s, t);
        if (st != KORE_OK) {
            if (st == KORE_ECUDA || st == KORE_ETIMEOUT) return st;   // the device is in doubt: stop
            r.sl[s].busy = false;
            r.sl[s].phase = 2;
            r.src->finished(t, st);
        }
    }
}

// The target of slot s has its eigenpairs in the device slot arrays: order them by
// `which`, copy them out, record its statistics and hand it back to the source.
int finish_target(Run &r, int s) {
    kore_plan *p = r.p;
    Ctx &c = r.c;
    Slot &x = r.sl[s];
    const EigsTarget &t = x.tgt;
    const kore_eps_opts &ot = t.opts;
    std::vector<double2> lam(std::max(x.nout, 1));
    IrState irs, irs0;
    if (x.nout > 0)
        KORE_CUDA_TRY(cudaMemcpyAsync(lam.data(), c.lam + s * kVecStride, x.nout * sizeof(double2),
                                      cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaMemcpyAsync(&irs, p->d_ir + s, sizeof(IrState), cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaMemcpyAsync(&irs0, p->d_ir, sizeof(IrState), cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    for (int k = 0; k < x.nout; ++k)
        if (!(std::isfinite(lam[k].x) && std::isfinite(lam[k].y))) {
            // B x = 0 or a NaN: keep the back-transformed Ritz value
            const double2 th = x.theta[k];
            const double d = th.x * th.x + th.y * th.y;
            const double2 sh = shift_of(ot);
            lam[k] = mk(sh.x + th.x / d, sh.y - th.y / d);
        }
    std::vector<int> order(x.nout);
    std::vector<double> key(x.nout);
    for (int k = 0; k < x.nout; ++k) {
        order[k] = k;
        key[k] = lambda_key(lam[k], ot.which, ot.target_re, ot.target_im);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    for (int k = 0; k < x.nout; ++k) {
        t.evals[2 * k] = lam[order[k]].x;
        t.evals[2 * k + 1] = lam[order[k]].y;
        if (t.evecs) {
            KORE_TRY(kore_scatter(p, x.Vt + (int64_t)order[k] * c.np, p->d_v[4]));
            KORE_CUDA_TRY(cudaMemcpyAsync(t.evecs + (size_t)k * 2 * p->n, p->d_v[4], p->n * sizeof(double2),
                                          cudaMemcpyDeviceToHost, p->stream));
        }
    }
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    if (t.nconv) *t.nconv = x.nconv;
    if (t.stats) {
        kore_stats &q = *t.stats;
        q = kore_stats{};
        q.nconv = x.nconv;
        q.restarts = x.restarts;
        q.op_applies = x.applies;
        q.refine_iters_max = irs.iters_max;
        q.solve_resid_max = irs.eta_max;
        q.sweeps = irs0.sweeps;   // sweep launches of the engine so far (counted in shift 0's state)
        q.iterate_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - r.t0).count();
        q.factor_reused = t.reused;
        q.warm_started = t.warm_started;
        q.shift_re = shift_of(ot).x;
        q.shift_im = shift_of(ot).y;
    }
    // the slot's warm vector for a later target: the sum of the eigenvectors just returned
    if (x.nout > 0 && x.nconv > 0 && s < p->warm_cap) {
        k_sum_cols<<<c.grid, 256, 0, p->stream>>>(c.np, x.Vt, x.nout, p->d_warm + (int64_t)s * c.np);
        k_unit<<<1, 1024, 0, p->stream>>>(c.np, p->d_warm + (int64_t)s * c.np);
        KORE_LAUNCHED(2);
        KORE_CUDA_TRY(cudaGetLastError());
        p->warm_ok[s] = 1;
    }
    x.busy = false;
    x.phase = 2;
    r.src->finished(t, irs.nan ? KORE_ENAN : (x.nconv == 0 ? KORE_ENOCONV : KORE_OK));
    return KORE_OK;
}

// Slot s has converged (or run out of restarts): form its Ritz vectors X = V Q Y in the
// restart buffer and start purifying them (or finish at once without pairs).
int begin_purify(Run &r, int s, const double2 *theta) {
    kore_plan *p = r.p;
    Ctx &c = r.c;
    Slot &x = r.sl[s];
    x.theta.assign(theta, theta + x.m);
    x.nout = std::min(x.nconv, x.tgt.max_pairs);
    if (x.nout == 0) return finish_target(r, s);
    TCols gc{};
    gc.mask = 1u << s;
    gc.n[s] = x.m; gc.j[s] = x.nout; gc.ld[s] = x.m;
    TVec a, b, d;
    for (int u = 0; u < kMaxTargets; ++u) a.p[u] = b.p[u] = d.p[u] = nullptr;
    // G = Q Y[:, 0:nout] (m x nout) into T's storage, then X = V G
    a.p[s] = c.Q + s * kSqStride; b.p[s] = c.Y + s * kSqStride; d.p[s] = c.Tm + s * kSqStride;
    k_gemm_vg<<<dim3(1, r.T), 256, 0, p->stream>>>(x.m, a, b, d, gc);
    a.p[s] = x.V; b.p[s] = c.Tm + s * kSqStride; d.p[s] = x.Vt;
    k_gemm_vg<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(c.np, a, b, d, gc);
    KORE_LAUNCHED(2);
    x.phase = 1;
    x.k = 0;
    x.pstep = 0;
    return KORE_OK;
}

// Eigenvector k of the slots in mask is final (purified): normalise it and take its
// eigenvalue as the FP64 least-squares Rayleigh quotient (B x)^H (A x) / ||B x||^2.
int finish_vectors(Run &r, const TVec &x, unsigned mask, const int *kidx) {
    kore_plan *p = r.p;
    Ctx &c = r.c;
    const int64_t np = c.np;
    TCols nc{};
    nc.mask = mask;
    k_nrm2_partial<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(np, x, c.dpart, mask);
    k_finish_col<<<r.T, 256, 0, p->stream>>>((int)c.grid, c.dpart, c.h, c.Hbar, c.beta, nc, 0);
    k_scale_copy<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(np, x, c.beta, x, mask);
    k_copy_vecs<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(np, x, contiguous(c.xin, r.T, np), mask);
    KORE_LAUNCHED(4);
    KORE_TRY(kore_spmv_a_shifts(p, c.xin, c.w, mask));
    KORE_TRY(kore_spmv_b_shifts(p, c.xin, c.t1, mask));
    k_rq_partial<<<dim3(c.grid, r.T), 256, 0, p->stream>>>(np, contiguous(c.w, r.T, np), contiguous(c.t1, r.T, np),
                                                          c.partial, mask);
    KORE_LAUNCHED(1);
    // k differs between slots: one finishing launch per distinct k
    unsigned left = mask;
    while (left) {
        const int s0 = __builtin_ctz(left);
        unsigned same = 0;
        for (int s = 0; s < r.T; ++s)
            if (((left >> s) & 1u) && kidx[s] == kidx[s0]) same |= 1u << s;
        k_rq_finish<<<r.T, 256, 0, p->stream>>>((int)c.grid, c.partial, c.lam, kidx[s0], same);
        KORE_LAUNCHED(1);
        left &= ~same;
    }
    return KORE_OK;
}

// The targets of kore_eigs_shifts: an array, each target's results at its index.
struct ArraySource : EigsSource {
    const kore_eps_opts *o;
    int ntarget, next_t = 0, max_pairs;
    int64_t n;
    double *evals, *evecs;
    int *nconv;
    kore_stats *st;
    bool nan = false, none = false;
    int err = KORE_OK;
    bool next(EigsTarget *t) override {
        if (next_t >= ntarget) return false;
        const int i = next_t++;
        t->opts = o[i];
        t->evals = evals + (size_t)2 * max_pairs * i;
        t->evecs = evecs ? evecs + (size_t)2 * n * max_pairs * i : nullptr;
        t->max_pairs = max_pairs;
        t->nconv = nconv + i;
        t->stats = st ? st + i : nullptr;
        return true;
    }
    void finished(const EigsTarget &, int status) override {
        if (status == KORE_ENAN) nan = true;
        else if (status == KORE_ENOCONV) none = true;
        else if (status != KORE_OK && err == KORE_OK) err = status;
    }
};

}  // namespace

// The batched shift-and-invert Krylov-Schur engine.  The plan's nshift factor slots
// run one target each; a free slot takes the source's next target (its shift is
// factorised there unless the slot holds it already), so targets that arrive while
// others run are admitted as slots free up.  Each target runs its own Krylov-Schur with
// its options.  One step applies OP once for every busy slot in shared launches (one
// multi-shift sparse product and one multi-shift sweep plus the FP64 refinement loop in
// mixed precision): an expanding slot extends its Arnoldi basis (batched Gram-Schmidt
// kernels follow), a purifying slot applies OP to its next Ritz vector.  A slot whose
// basis is full gets its projected Schur problem (one CTA per such slot), its
// convergence test and its thick restart independently of the others.  A target's
// arithmetic does not depend on the other slots: every kernel works per shift and
// reduces in a fixed order.
int kore_eigs_engine(kore_plan *p, EigsSource *src, bool *valid, int max_ncv) {
    const int T = p->nshift;
    if (!p->factored) return KORE_ENOTFACTORED;
    if (!p->has_b || !src || T < 1 || T > kMaxTargets || max_ncv < 2 || max_ncv > kMaxNcv) return KORE_EINVAL;
    const int64_t np = p->np;
    const int M = max_ncv;   // every slot's basis holds M + 1 columns
    const int64_t vcols = (int64_t)T * (M + 1);
    if (p->ks_cap < vcols) {
        cudaFree(p->d_V); cudaFree(p->d_Vtmp); cudaFree(p->d_ksx);
        p->d_V = p->d_Vtmp = p->d_ksx = nullptr;
        p->ks_cap = 0;
        KORE_TRY(kore_alloc(p, (void **)&p->d_V, (size_t)np * vcols * sizeof(double2)));
        KORE_TRY(kore_alloc(p, (void **)&p->d_Vtmp, (size_t)np * vcols * sizeof(double2)));
        KORE_TRY(kore_alloc(p, (void **)&p->d_ksx, (size_t)np * T * sizeof(double2)));
        p->ks_cap = vcols;
    }
    if (p->warm_cap < T) {
        cudaFree(p->d_warm);
        p->d_warm = nullptr;
        p->warm_cap = 0;
        p->warm_ok.assign(T, 0);
        KORE_TRY(kore_alloc(p, (void **)&p->d_warm, (size_t)np * T * sizeof(double2)));
        p->warm_cap = T;
    }
    if (p->ks_small_cap < T) {
        cudaFree(p->d_small);
        p->d_small = nullptr;
        p->ks_small_cap = 0;
        KORE_TRY(kore_alloc(p, (void **)&p->d_small, small_elems(T) * sizeof(double2)));
        p->ks_small_cap = T;
    }
    Run r;
    r.p = p; r.T = T; r.M = M; r.src = src;
    r.t0 = std::chrono::steady_clock::now();
    Ctx &c = r.c;
    c.p = p; c.T = T; c.np = np;
    c.grid = std::min<unsigned>(kore_div_up(np, 256), 2u * p->num_sms);
    if (c.grid > (unsigned)kGridMax) return KORE_EINVAL;
    c.t1 = p->d_bb; c.w = p->d_xb; c.xin = p->d_ksx;
    carve_small(c, p->d_small);
    c.applies.assign(T, 0);
    r.sl.assign(T, Slot{});
    for (int s = 0; s < T; ++s) {
        r.sl[s].V = p->d_V + (int64_t)s * (M + 1) * np;
        r.sl[s].Vt = p->d_Vtmp + (int64_t)s * (M + 1) * np;
        r.sl[s].valid = valid && valid[s];
    }
    KORE_TRY(kore_ir_reset(p));
    KORE_TRY(kore_allow_max_dyn_smem(k_schur, p->device));
    r.sb.hstride = kHbarStride; r.sb.sqstride = kSqStride; r.sb.vstride = kVecStride;
    const SchurOut so{c.Tm, c.Q, c.Y, c.theta, c.est, c.bnew, c.info};
    std::vector<double> h_est((size_t)T * kVecStride);
    std::vector<double2> h_theta((size_t)T * kVecStride);
    std::vector<int> h_info(T);
    std::vector<double> tols(T);
    std::vector<int> kidx(T);
    const bool mixed = p->prec == KORE_PREC_MIXED;

    for (;;) {
        KORE_TRY(fill_slots(r));
        unsigned expm = 0, purm = 0;
        for (int s = 0; s < T; ++s) {
            if (r.sl[s].phase == 0) expm |= 1u << s;
            else if (r.sl[s].phase == 1) purm |= 1u << s;
        }
        if (!(expm | purm)) break;
        // Each OP application of an expanding slot is refined to 1e-16 unless the
        // target asks otherwise.  Measured on the 240k shell: at 1e-14 the mixed path's
        // eigen residuals were ten times the FP64 path's and ill-conditioned eigenvalues
        // drifted further than a rounding-level perturbation of A moves them; at 1e-15
        // that held at 0.5i but not at 0.46i (residuals 30 times the FP64 path's); at
        // 1e-16 the residuals are at or below the FP64 path's at every target tried, for
        // about 5% more sweeps.  The accuracy has to come from the Krylov phase:
        // purification amplifies the components of eigenvalues nearer the target than
        // the pair's own, so it cannot repair a pair.  A purifying application is refined
        // until its residual stops decreasing.
        TVec vin, vb;
        TCols tc{};
        tc.mask = expm;
        for (int u = 0; u < kMaxTargets; ++u) vin.p[u] = vb.p[u] = nullptr;
        for (int s = 0; s < T; ++s) {
            Slot &x = r.sl[s];
            vb.p[s] = x.V;
            vin.p[s] = (x.phase == 1) ? x.Vt + (int64_t)x.k * np : x.V + (int64_t)x.j * np;
            tc.n[s] = x.j + 1; tc.j[s] = x.j; tc.ld[s] = x.m + 1;
            const double rt = (x.busy && x.tgt.opts.refine_tol > 0.0) ? x.tgt.opts.refine_tol : kEigsRefineTol;
            tols[s] = (x.phase == 1 && mixed) ? kFloorRefineTol : rt;
            kidx[s] = x.k;
        }
        c.refine_tol = kEigsRefineTol;
        // a purifying slot with purify = 0 skips the application
        unsigned appm = expm;
        for (int s = 0; s < T; ++s)
            if (((purm >> s) & 1u) && r.sl[s].tgt.opts.purify > 0) appm |= 1u << s;
        if (appm) KORE_TRY(apply_op(c, vin, appm, tols.data()));
        for (int s = 0; s < T; ++s)
            if ((appm >> s) & 1u) r.sl[s].applies += 1;
        if (expm) KORE_TRY(orthonormalise(c, vb, tc));
        if (purm) {
            // x <- OP x for the purifying slots that applied it; a vector is final after
            // opts.purify applications
            unsigned app_p = appm & purm, fin = 0;
            k_copy_vecs<<<dim3(c.grid, T), 256, 0, p->stream>>>(np, contiguous(c.w, T, np), vin, app_p);
            KORE_LAUNCHED(1);
            for (int s = 0; s < T; ++s)
                if ((purm >> s) & 1u) {
                    Slot &x = r.sl[s];
                    if ((app_p >> s) & 1u) x.pstep += 1;
                    if (x.pstep >= x.tgt.opts.purify) fin |= 1u << s;
                }
            if (fin) KORE_TRY(finish_vectors(r, vin, fin, kidx.data()));
            for (int s = 0; s < T; ++s)
                if ((fin >> s) & 1u) {
                    Slot &x = r.sl[s];
                    x.k += 1;
                    x.pstep = 0;
                    if (x.k == x.nout) KORE_TRY(finish_target(r, s));
                }
        }
        unsigned full = 0;
        for (int s = 0; s < T; ++s)
            if ((expm >> s) & 1u) {
                r.sl[s].j += 1;
                if (r.sl[s].j == r.sl[s].m) full |= 1u << s;
            }
        if (!full) continue;
        // projected Schur problems of the slots whose basis is full
        const size_t schur_smem = (size_t)3 * M * M * sizeof(double2);
        if (p->prof) KORE_TRY(kore_prof_mark(p, 4, true));
        r.sb.mask = full;
        k_schur<<<T, kSchurT, schur_smem, p->stream>>>(c.Hbar, r.sb, so);
        KORE_LAUNCHED(1);
        KORE_CUDA_TRY(cudaGetLastError());
        if (p->prof) KORE_TRY(kore_prof_mark(p, 4, false));
        KORE_CUDA_TRY(cudaMemcpyAsync(h_est.data(), c.est, h_est.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                      p->stream));
        KORE_CUDA_TRY(cudaMemcpyAsync(h_theta.data(), c.theta, h_theta.size() * sizeof(double2),
                                      cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaMemcpyAsync(h_info.data(), c.info, T * sizeof(int), cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
        KORE_TRY(kore_check_device_error(p));
        // convergence tests and thick restarts
        TCols rc{};
        TVec rV, rQ, rOut, rSrc, rDst;
        for (int u = 0; u < kMaxTargets; ++u) rV.p[u] = rQ.p[u] = rOut.p[u] = rSrc.p[u] = rDst.p[u] = nullptr;
        for (int s = 0; s < T; ++s) {
            if (!((full >> s) & 1u)) continue;
            Slot &x = r.sl[s];
            const kore_eps_opts &ot = x.tgt.opts;
            x.restarts += 1;
            if (h_info[s] != 0) {
                x.nconv = 0;
                KORE_TRY(begin_purify(r, s, h_theta.data() + (size_t)s * kVecStride));
                continue;
            }
            const double *est = h_est.data() + (size_t)s * kVecStride;
            int ncv = 0;
            while (ncv < x.m && est[ncv] < ot.tol) ++ncv;
            x.nconv = ncv;
            if (ncv >= x.nev || x.restarts >= ot.maxit) {
                KORE_TRY(begin_purify(r, s, h_theta.data() + (size_t)s * kVecStride));
                continue;
            }
            const int l = std::max(1, (x.m - ncv) / 2);
            const int keep = std::min(ncv + l, x.m - 1);
            rc.mask |= 1u << s;
            rc.n[s] = x.m; rc.j[s] = keep; rc.ld[s] = x.m;
            rV.p[s] = x.V; rQ.p[s] = c.Q + s * kSqStride; rOut.p[s] = x.Vt;
            rSrc.p[s] = x.V + (int64_t)x.m * np; rDst.p[s] = x.Vt + (int64_t)keep * np;
        }
        if (rc.mask) {
            if (p->prof) KORE_TRY(kore_prof_mark(p, 4, true));
            k_gemm_vg<<<dim3(c.grid, T), 256, 0, p->stream>>>(np, rV, rQ, rOut, rc);
            k_copy_vecs<<<dim3(c.grid, T), 256, 0, p->stream>>>(np, rSrc, rDst, rc.mask);
            TCols hc = rc;
            for (int s = 0; s < T; ++s) { hc.n[s] = rc.j[s]; hc.ld[s] = r.sl[s].m + 1; }
            k_restart_h<<<T, 256, 0, p->stream>>>(c.Tm, c.bnew, c.Hbar, hc);
            KORE_LAUNCHED(3);
            if (p->prof) KORE_TRY(kore_prof_mark(p, 4, false));
            for (int s = 0; s < T; ++s)
                if ((rc.mask >> s) & 1u) {
                    std::swap(r.sl[s].V, r.sl[s].Vt);
                    r.sl[s].j = rc.j[s];
                }
        }
    }
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    if (valid)
        for (int s = 0; s < T; ++s) valid[s] = r.sl[s].valid;
    return kore_check_device_error(p);
}

// kore_eigs / kore_eigs_shifts: targets 0 .. nshift-1 are the factorised shifts, the
// others are admitted into slots as earlier ones finish.
int kore_eigs_impl(kore_plan *p, int ntarget, const kore_eps_opts *o, double *evals, double *evecs, int max_pairs,
                   int *nconv_out, kore_stats *st) {
    if (!p->factored) return KORE_ENOTFACTORED;
    const int T = p->nshift;
    if (!o || T < 1 || T > kMaxTargets || ntarget < T) return KORE_EINVAL;
    for (int t = 0; t < ntarget; ++t) {
        KORE_TRY(check_opts(p, o[t], kMaxNcv));
        if (t < T && (shift_of(o[t]).x != p->sigmas[t].x || shift_of(o[t]).y != p->sigmas[t].y)) return KORE_EINVAL;
    }
    ArraySource src;
    src.o = o; src.ntarget = ntarget; src.max_pairs = max_pairs; src.n = p->n;
    src.evals = evals; src.evecs = evecs; src.nconv = nconv_out; src.st = st;
    bool valid[kMaxTargets];
    for (int s = 0; s < kMaxTargets; ++s) valid[s] = s < T;
    int M = 2;
    for (int t = 0; t < ntarget; ++t) M = std::max(M, ncv_of(p, o[t]));
    const int rc = kore_eigs_engine(p, &src, valid, M);
    if (rc != KORE_OK) return rc;
    if (src.err != KORE_OK) return src.err;
    if (src.nan) return KORE_ENAN;
    return src.none ? KORE_ENOCONV : KORE_OK;
}
