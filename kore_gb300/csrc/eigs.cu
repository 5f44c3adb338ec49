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
// The dimension defaults follow SLEPc: ncv = min(n, max(2 nev, nev + 15)).
#include "kore_internal.cuh"
#include <cmath>
#include <algorithm>
#include <chrono>
#include <vector>

namespace {

constexpr int kMaxNcv = 64;

// ----------------------------------------------------------------------------- sort keys
// Ascending key = wanted first (the comparison functions of SLEPc's `which`).
__host__ __device__ inline double which_key(double2 theta, int which, double tre, double tim) {
    // lambda = tau + 1/theta
    const double d = theta.x * theta.x + theta.y * theta.y;
    double lre, lim;
    if (d > 0.0) { lre = tre + theta.x / d; lim = tim - theta.y / d; }
    else { lre = INFINITY; lim = 0.0; }
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

// One CTA of 128 threads (four warps, one per SM sub-partition, so the FP64 updates
// of a rotation run on all four FP64 pipes).  Hbar: (m+1) x m column-major (ld m+1);
// row m is the residual row.
constexpr int kSchurT = 128;
__global__ void __launch_bounds__(kSchurT) k_schur(const double2 *__restrict__ Hbar, int m, int which, double tre,
                                                   double tim, SchurOut out) {
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
    for (int j = tid; j < m; j += kSchurT) key[j] = which_key(H[j + j * m], which, tre, tim);
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
// partial[b*nc + c] = sum over the CTA's rows of conj(V[:,c]) w for c < ncol, and, with
// with_norm, entry c = ncol = sum |w|^2 (nc = ncol + with_norm).  run (may be null):
// the kernel returns at once unless *run != 0.
constexpr int kDotThreads = 256;
constexpr int kDotChunk = 8;

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
__global__ void __launch_bounds__(kDotThreads) k_mdot(int64_t np, int ncol, const double2 *__restrict__ V,
                                                      const double2 *__restrict__ w, double2 *__restrict__ partial,
                                                      int with_norm, const int *__restrict__ run) {
    if (run && *run == 0) return;
    __shared__ double sm[kDotThreads / 32][2 * kDotChunk];
    const int nc = ncol + with_norm;
    for (int c0 = 0; c0 < nc; c0 += kDotChunk) {
        double2 acc[kDotChunk];
#pragma unroll
        for (int t = 0; t < kDotChunk; ++t) acc[t] = mk(0.0, 0.0);
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
            const double2 wr = w[r];
#pragma unroll
            for (int t = 0; t < kDotChunk; ++t)
                if (c0 + t < nc) acc[t] = cfmaconj(acc[t], (c0 + t < ncol) ? V[r + (int64_t)(c0 + t) * np] : wr, wr);
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

// h[c] (+)= sum_b partial[b*ncol + c] (one CTA per c); returns at once unless *run != 0
__global__ void k_mdot_reduce(int nblk, int ncol, const double2 *__restrict__ partial, double2 *__restrict__ h,
                              int accumulate, const int *__restrict__ run) {
    if (run && *run == 0) return;
    const int c = blockIdx.x;
    double2 s = mk(0.0, 0.0);
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) s = s + partial[(int64_t)b * ncol + c];
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

// w -= V h  (ncol columns); h is this pass's coefficients; returns at once unless *run != 0
__global__ void k_mgs_update(int64_t np, int ncol, const double2 *__restrict__ V, const double2 *__restrict__ h,
                             double2 *__restrict__ w, const int *__restrict__ run) {
    if (run && *run == 0) return;
    __shared__ double2 hs[kMaxNcv + 1];
    for (int c = threadIdx.x; c < ncol; c += blockDim.x) hs[c] = h[c];
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
        double2 acc = w[r];
        for (int c = 0; c < ncol; ++c) acc = cfms(acc, V[r + (int64_t)c * np], hs[c]);
        w[r] = acc;
    }
}

// partial sums of |w|^2
__global__ void k_nrm2_partial(int64_t np, const double2 *__restrict__ w, double *__restrict__ partial) {
    double s = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x)
        s += abs2(w[r]);
    s = warp_sum_d(s);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t += sm[wv];
        partial[blockIdx.x] = t;
    }
}
// Refinement decision of classical Gram-Schmidt (SLEPc's default, refinement "if needed"
// with eta = 1/sqrt(2)): h1[ncol].x = ||w||^2 before the first pass; the norm after it
// is sqrt(||w||^2 - sum |h1_c|^2) (exact for orthonormal V); a second pass runs when
// that is below eta ||w||.  Clears h2, which a skipped second pass leaves untouched.
__global__ void k_refine_decide(const double2 *__restrict__ h1, int ncol, double2 *__restrict__ h2,
                                int *__restrict__ run2) {
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
        *run2 = (onrm2 - t < 0.5 * onrm2) ? 1 : 0;
    }
}

// beta = sqrt(sum partial); Hbar[j+1 + j*ld] = beta; h (ncol entries) copied into Hbar column j
__global__ void k_finish_col(int nblk, const double *__restrict__ partial, const double2 *__restrict__ h, int ncol,
                             double2 *__restrict__ Hbar, int ld, int j, double *__restrict__ beta_out) {
    __shared__ double sm[32];
    double s = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += partial[b];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t += sm[wv];
        const double beta = sqrt(t);
        *beta_out = beta;
        if (j >= 0) Hbar[(j + 1) + (int64_t)j * ld] = mk(beta, 0.0);
    }
    if (j >= 0)
        for (int c = threadIdx.x; c < ncol; c += blockDim.x) Hbar[c + (int64_t)j * ld] = h[c];
}
// dst = src / *scal (scal > 0), or dst = src * (1/||src||) by passing norm
__global__ void k_scale_copy(int64_t np, const double2 *__restrict__ src, const double *__restrict__ scal,
                             double2 *__restrict__ dst) {
    const double s = *scal;
    const double inv = (s > 0.0) ? 1.0 / s : 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x)
        dst[r] = inv * src[r];
}

// Vout[:, c] = V[:, 0:m] G[:, c] for c < ncol; G is m x ncol column-major (ld m)
constexpr int kGemmChunk = 8;
__global__ void k_gemm_vg(int64_t np, int m, int ncol, const double2 *__restrict__ V, const double2 *__restrict__ G,
                          int ldg, double2 *__restrict__ Vout) {
    __shared__ double2 gs[kMaxNcv * kGemmChunk];
    for (int c0 = 0; c0 < ncol; c0 += kGemmChunk) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < m * kGemmChunk; idx += blockDim.x) {
            const int j = idx % m, t = idx / m;
            gs[j * kGemmChunk + t] = (c0 + t < ncol) ? G[j + (int64_t)(c0 + t) * ldg] : mk(0.0, 0.0);
        }
        __syncthreads();
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < np; r += (int64_t)gridDim.x * blockDim.x) {
            double2 acc[kGemmChunk];
#pragma unroll
            for (int t = 0; t < kGemmChunk; ++t) acc[t] = mk(0.0, 0.0);
            for (int j = 0; j < m; ++j) {
                const double2 v = V[r + (int64_t)j * np];
#pragma unroll
                for (int t = 0; t < kGemmChunk; ++t) acc[t] = cfma(acc[t], v, gs[j * kGemmChunk + t]);
            }
#pragma unroll
            for (int t = 0; t < kGemmChunk; ++t)
                if (c0 + t < ncol) Vout[r + (int64_t)(c0 + t) * np] = acc[t];
        }
    }
}

// Hbar <- [T[0:p,0:p]; bnew[0:p]] (ld m+1), other entries zero
__global__ void k_restart_h(int m, int p, const double2 *__restrict__ T, const double2 *__restrict__ bnew,
                            double2 *__restrict__ Hbar) {
    const int ld = m + 1;
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

// ----------------------------------------------------------------------------- host helpers
struct Ctx {
    kore_plan *p;
    int64_t np;
    unsigned grid;
    double2 *V, *Vtmp, *w, *t1;
    double2 *Hbar, *partial, *h;
    double *dpart, *beta;
    int *run2;          // second Gram-Schmidt pass needed (device flag)
    double refine_tol;
};

// Deterministic complex standard normal start vector (SplitMix64 + Box-Muller).
static uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static void start_vector(int64_t n, uint64_t seed, std::vector<double2> &v) {
    v.resize(n);
    uint64_t s = seed;
    const double two_pi = 6.283185307179586476925286766559;
    for (int64_t i = 0; i < n; ++i) {
        double u1 = ((splitmix(s) >> 11) + 1) * (1.0 / 9007199254740993.0);
        double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
        double r = std::sqrt(-2.0 * std::log(u1));
        v[i] = mk(r * std::cos(two_pi * u2), r * std::sin(two_pi * u2));
    }
}

int apply_op(Ctx &c, const double2 *v, double2 *out) {
    KORE_TRY(kore_spmv_b(c.p, v, c.t1));
    return kore_apply_inverse(c.p, c.t1, out, c.refine_tol);
}

// orthogonalise w against V[:, 0:ncol] twice, write h and beta into Hbar column j,
// v_{j+1} = w / beta
int orthonormalise(Ctx &c, int ncol, int j, int ldh) {
    kore_plan *p = c.p;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 3, true));
    // first pass, with ||w||^2 as entry ncol of h1
    double2 *h1 = c.h, *h2 = c.h + kMaxNcv + 1;
    k_mdot<<<c.grid, kDotThreads, 0, p->stream>>>(c.np, ncol, c.V, c.w, c.partial, 1, nullptr);
    k_mdot_reduce<<<ncol + 1, 256, 0, p->stream>>>((int)c.grid, ncol + 1, c.partial, h1, 0, nullptr);
    k_mgs_update<<<c.grid, 256, 0, p->stream>>>(c.np, ncol, c.V, h1, c.w, nullptr);
    k_refine_decide<<<1, 256, 0, p->stream>>>(h1, ncol, h2, c.run2);
    // second pass if needed
    k_mdot<<<c.grid, kDotThreads, 0, p->stream>>>(c.np, ncol, c.V, c.w, c.partial, 0, c.run2);
    k_mdot_reduce<<<ncol, 256, 0, p->stream>>>((int)c.grid, ncol, c.partial, h2, 0, c.run2);
    k_mgs_update<<<c.grid, 256, 0, p->stream>>>(c.np, ncol, c.V, h2, c.w, c.run2);
    KORE_LAUNCHED(7);
    // h = h1 + h2
    k_mdot_reduce<<<ncol, 32, 0, p->stream>>>(1, ncol, h2, h1, 1, nullptr);
    k_nrm2_partial<<<c.grid, 256, 0, p->stream>>>(c.np, c.w, c.dpart);
    k_finish_col<<<1, 256, 0, p->stream>>>((int)c.grid, c.dpart, c.h, ncol, c.Hbar, ldh, j, c.beta);
    k_scale_copy<<<c.grid, 256, 0, p->stream>>>(c.np, c.w, c.beta, c.V + (int64_t)(j + 1) * c.np);
    KORE_LAUNCHED(4);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 3, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

}  // namespace

int kore_eigs_impl(kore_plan *p, const kore_eps_opts *o, double *evals, double *evecs, int max_pairs, int *nconv_out,
                   kore_stats *st) {
    if (!p->factored) return KORE_ENOTFACTORED;
    if (!p->has_b || !o || o->nev <= 0 || o->which < 0 || o->which > 8) return KORE_EINVAL;
    if (o->target_re != p->sigma_re || o->target_im != p->sigma_im) return KORE_EINVAL;
    const int64_t n = p->n, np = p->np;
    const int nev = o->nev;
    int m = o->ncv > 0 ? o->ncv : (int)std::min<int64_t>(n, std::max(2 * nev, nev + 15));
    if (m > kMaxNcv || m <= nev || m > n) return KORE_EINVAL;
    auto t0 = std::chrono::steady_clock::now();
    if (st) *st = kore_stats{};

    // workspace
    if (p->ks_cap < m + 1) {
        cudaFree(p->d_V); cudaFree(p->d_Vtmp);
        p->d_V = p->d_Vtmp = nullptr;
        KORE_TRY(kore_alloc(p, (void **)&p->d_V, (size_t)np * (m + 1) * sizeof(double2)));
        KORE_TRY(kore_alloc(p, (void **)&p->d_Vtmp, (size_t)np * (m + 1) * sizeof(double2)));
        p->ks_cap = m + 1;
    }
    if (!p->d_small) {
        // Hbar, T, Q, Y, theta, est, bnew, h(2x), partial, dpart, beta, info
        const size_t sz = (size_t)(kMaxNcv + 1) * kMaxNcv * 4 + 8 * (kMaxNcv + 1) + 2048 * (kMaxNcv + 1) + 4096;
        KORE_TRY(kore_alloc(p, (void **)&p->d_small, sz * sizeof(double2)));
    }
    double2 *base = p->d_small;
    const int ldh = m + 1;
    Ctx c;
    c.p = p; c.np = np;
    c.grid = std::min<unsigned>(kore_div_up(np, 256), 2u * p->num_sms);
    c.V = p->d_V; c.Vtmp = p->d_Vtmp; c.w = p->d_v[2]; c.t1 = p->d_v[3];
    c.Hbar = base;
    double2 *dT = base + (kMaxNcv + 1) * kMaxNcv;
    double2 *dQ = dT + kMaxNcv * kMaxNcv;
    double2 *dY = dQ + kMaxNcv * kMaxNcv;
    double2 *dtheta = dY + kMaxNcv * kMaxNcv;
    double2 *dbnew = dtheta + (kMaxNcv + 1);
    c.h = dbnew + (kMaxNcv + 1);                    // 2 x (kMaxNcv+1)
    double *dest = reinterpret_cast<double *>(c.h + 2 * (kMaxNcv + 1));   // kMaxNcv+1 doubles
    c.partial = c.h + 3 * (kMaxNcv + 1);             // grid x ncol
    c.dpart = reinterpret_cast<double *>(c.partial + 2048 * (kMaxNcv + 1));
    c.beta = c.dpart + 2048;
    int *dinfo = reinterpret_cast<int *>(c.beta + 8);
    c.run2 = dinfo + 4;
    if (c.grid > 2048) return KORE_EINVAL;

    // start vector
    std::vector<double2> hv;
    start_vector(n, o->seed, hv);
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_v[4], hv.data(), n * sizeof(double2), cudaMemcpyHostToDevice, p->stream));
    KORE_TRY(kore_gather(p, p->d_v[4], c.w));
    k_nrm2_partial<<<c.grid, 256, 0, p->stream>>>(np, c.w, c.dpart);
    k_finish_col<<<1, 256, 0, p->stream>>>((int)c.grid, c.dpart, c.h, 0, c.Hbar, ldh, -1, c.beta);
    k_scale_copy<<<c.grid, 256, 0, p->stream>>>(np, c.w, c.beta, c.V);
    KORE_LAUNCHED(3);
    KORE_CUDA_TRY(cudaMemsetAsync(c.Hbar, 0, sizeof(double2) * ldh * m, p->stream));

    const size_t schur_smem = (size_t)3 * m * m * sizeof(double2);
    KORE_TRY(kore_allow_max_dyn_smem(k_schur, p->device));
    std::vector<double> h_est(m);
    std::vector<double2> h_theta(m);
    int h_info = 0;
    int kkeep = 0, nconv = 0, restarts = 0;
    c.refine_tol = o->refine_tol;
    KORE_TRY(kore_ir_reset(p));
    for (restarts = 0;; ++restarts) {
        // Arnoldi expansion kkeep .. m-1
        for (int j = kkeep; j < m; ++j) {
            KORE_TRY(apply_op(c, c.V + (int64_t)j * np, c.w));
            KORE_TRY(orthonormalise(c, j + 1, j, ldh));
        }
        if (p->prof) KORE_TRY(kore_prof_mark(p, 4, true));
        SchurOut so{dT, dQ, dY, dtheta, dest, dbnew, dinfo};
        k_schur<<<1, kSchurT, schur_smem, p->stream>>>(c.Hbar, m, o->which, o->target_re, o->target_im, so);
        KORE_LAUNCHED(1);
        KORE_CUDA_TRY(cudaGetLastError());
        if (p->prof) KORE_TRY(kore_prof_mark(p, 4, false));
        KORE_CUDA_TRY(cudaMemcpyAsync(h_est.data(), dest, m * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaMemcpyAsync(h_theta.data(), dtheta, m * sizeof(double2), cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaMemcpyAsync(&h_info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
        KORE_TRY(kore_check_device_error(p));
        if (h_info != 0) return KORE_ENOCONV;
        nconv = 0;
        while (nconv < m && h_est[nconv] < o->tol) ++nconv;
        if (nconv >= nev || restarts + 1 >= o->maxit) break;
        // thick restart
        const int l = std::max(1, (m - nconv) / 2);
        const int keep = std::min(nconv + l, m - 1);
        if (p->prof) KORE_TRY(kore_prof_mark(p, 4, true));
        k_gemm_vg<<<c.grid, 256, 0, p->stream>>>(np, m, keep, c.V, dQ, m, c.Vtmp);
        KORE_CUDA_TRY(cudaMemcpyAsync(c.Vtmp + (int64_t)keep * np, c.V + (int64_t)m * np, np * sizeof(double2),
                                      cudaMemcpyDeviceToDevice, p->stream));
        k_restart_h<<<1, 256, 0, p->stream>>>(m, keep, dT, dbnew, c.Hbar);
        KORE_LAUNCHED(2);
        if (p->prof) KORE_TRY(kore_prof_mark(p, 4, false));
        std::swap(c.V, c.Vtmp);
        kkeep = keep;
    }
    // keep the plan's pointers consistent with the swapped buffers
    p->d_V = c.V;
    p->d_Vtmp = c.Vtmp;
    const int nout = std::min(nconv, max_pairs);
    // eigenvalues in Schur order (already sorted by `which`)
    for (int j = 0; j < nout; ++j) {
        const double2 th = h_theta[j];
        const double d = th.x * th.x + th.y * th.y;
        evals[2 * j] = o->target_re + th.x / d;
        evals[2 * j + 1] = o->target_im - th.y / d;
    }
    if (evecs && nout > 0) {
        // Ritz vectors X = V Q Y[:, 0:nout]: G = Q Y (m x nout) on the device, then V G
        // G computed column by column with the tall-skinny kernel on the small matrices
        double2 *G = dT;  // reuse T storage: m x nout
        k_gemm_vg<<<1, 256, 0, p->stream>>>(m, m, nout, dQ, dY, m, G);
        k_gemm_vg<<<c.grid, 256, 0, p->stream>>>(np, m, nout, c.V, G, m, c.Vtmp);
        KORE_LAUNCHED(2);
        for (int j = 0; j < nout; ++j) {
            double2 *x = c.Vtmp + (int64_t)j * np;
            if (o->purify) {
                KORE_TRY(apply_op(c, x, c.w));
                KORE_CUDA_TRY(cudaMemcpyAsync(x, c.w, np * sizeof(double2), cudaMemcpyDeviceToDevice, p->stream));
            }
            k_nrm2_partial<<<c.grid, 256, 0, p->stream>>>(np, x, c.dpart);
            k_finish_col<<<1, 256, 0, p->stream>>>((int)c.grid, c.dpart, c.h, 0, c.Hbar, ldh, -1, c.beta);
            k_scale_copy<<<c.grid, 256, 0, p->stream>>>(np, x, c.beta, c.w);
            KORE_LAUNCHED(3);
            KORE_TRY(kore_scatter(p, c.w, p->d_v[4]));
            KORE_CUDA_TRY(cudaMemcpyAsync(evecs + 2 * n * (int64_t)j, p->d_v[4], n * sizeof(double2),
                                          cudaMemcpyDeviceToHost, p->stream));
        }
    }
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    KORE_TRY(kore_check_device_error(p));
    *nconv_out = nconv;
    IrState irs;
    KORE_TRY(kore_ir_read(p, &irs));
    if (irs.nan) return KORE_ENAN;
    if (st) {
        st->nconv = nconv;
        st->restarts = restarts + 1;
        st->op_applies = (p->prec == KORE_PREC_MIXED) ? irs.applies : irs.sweeps;
        st->sweeps = irs.sweeps;
        st->refine_iters_max = irs.iters_max;
        st->solve_resid_max = irs.eta_max;
        st->iterate_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return nconv > 0 ? KORE_OK : KORE_ENOCONV;
}
