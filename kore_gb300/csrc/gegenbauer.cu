// Multiplication operators of the Gegenbauer (ultraspherical) basis on the GPU.
//
// kore's submatrices.py builds every radial operator r^X D^Y of the tau method as
// G * M(S r^X, Y) * D_Y, where M(a, lam) multiplies a C^(lam) series by the function
// whose C^(lam) coefficients are a (Mlam, bin/utils.py:962-1051).  The entries of M
// follow from the linearisation of products of ultraspherical polynomials
// (Olver & Townsend, SIAM Review 55, 2013):
//     M[j, k] = sum_{s = s0}^{k} a[2 s + j - k] c_s(k, |j - k|),   s0 = max(0, k - j),
// with c_{s0} in closed form and c_{s+1} / c_s a rational function of (s, j, k, lam).
// lam = 0 (Chebyshev T) is the Toeplitz-plus-Hankel form 0.5 (a[|j-k|] + a[j+k]) with
// a[0] doubled and the Hankel part absent in row 0.
//
// One thread per band entry (row j, diagonal d): N (2h + 1) independent FP64 sums of
// at most N terms, a few microseconds for the sizes kore uses (N <= 1024).
#include "kore_internal.cuh"

namespace {

// closed form of c_s(j, k) (the first coefficient of the recurrence)
__device__ double lin_coeff_first(int s, double lam, int j, int k) {
    double p1 = 1.0, p3 = 1.0, p2 = 1.0, p4 = 1.0;
    for (int t = 0; t < s; ++t) {
        p1 = p1 * (lam + t) / (double)(1 + t);
        p3 = p3 * (2.0 * lam + j + k - 2 * s + t) / (lam + j + k - 2 * s + t);
    }
    for (int t = 0; t < j - s; ++t) {
        p2 = p2 * (lam + t) / (double)(1 + t);
        p4 = p4 * (double)(k - s + 1 + t) / (k - s + lam + t);
    }
    return p1 * p2 * p3 * p4 * (j + k + lam - 2.0 * s) / (j + k + lam - s);
}

// band[(d + h) N + j] = M[j, j + d] for |d| <= h (0 outside the matrix)
__global__ void k_gegen_mult(int N, const double *__restrict__ a, double lam, int h, double *__restrict__ band) {
    const int64_t total = (int64_t)N * (2 * h + 1);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % N), d = (int)(idx / N) - h, k = j + d;
        double v = 0.0;
        if (k >= 0 && k < N) {
            auto coef = [&](int i) { return (i >= 0 && i < N) ? a[i] : 0.0; };
            if (lam == 0.0) {
                const int dj = (j > k) ? j - k : k - j;
                const double t = (dj == 0) ? 2.0 * a[0] : a[dj];
                const double hk = (j >= 1 && j + k < N) ? ((j + k == 0) ? 2.0 * a[0] : a[j + k]) : 0.0;
                v = 0.5 * (t + hk);
            } else {
                const int s0 = (k - j > 0) ? k - j : 0;
                const int kk0 = (j > k) ? j - k : k - j;
                double c = lin_coeff_first(s0, lam, k, kk0);
                double acc = coef(2 * s0 + j - k) * c;
                const double jf = (double)k;
                double s = (double)s0, kc = (double)kk0;
                for (int step = 1; step < k - s0 + 1; ++step) {
                    const double t1 = (jf + kc + lam - s) * (lam + s) * (jf - s) * (2.0 * lam + jf + kc - s) * (kc - s + lam);
                    const double t2 = (jf + kc + lam - s + 1.0) * (s + 1.0) * (lam + jf - s - 1.0) * (lam + jf + kc - s) *
                                      (kc - s + 1.0);
                    c = c * t1 / t2;
                    s += 1.0;
                    kc += 2.0;
                    acc = acc + coef((int)(2.0 * s) + j - k) * c;
                }
                v = acc;
            }
        }
        band[idx] = v;
    }
}

}  // namespace

extern "C" int kore_gegenbauer_mult(int device, int N, const double *a0, double lam, int h, double *band) {
    if (N <= 0 || N > 8192 || !a0 || !band || h < 0 || h >= N || !(lam >= 0.0)) return KORE_EINVAL;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device) KORE_CUDA_TRY(cudaSetDevice(device));
    const size_t nb = (size_t)N * (2 * h + 1);
    double *da = nullptr, *db = nullptr;
    int rc = KORE_OK;
    auto ck = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == KORE_OK) rc = (e == cudaErrorMemoryAllocation) ? KORE_ENOMEM : KORE_ECUDA;
    };
    ck(cudaMalloc(&da, N * sizeof(double)));
    ck(cudaMalloc(&db, nb * sizeof(double)));
    if (rc == KORE_OK) {
        ck(cudaMemcpy(da, a0, N * sizeof(double), cudaMemcpyHostToDevice));
        k_gegen_mult<<<kore_div_up((long long)nb, 128), 128>>>(N, da, lam, h, db);
        KORE_LAUNCHED(1);
        ck(cudaGetLastError());
        ck(cudaMemcpy(band, db, nb * sizeof(double), cudaMemcpyDeviceToHost));
    }
    cudaFree(da);
    cudaFree(db);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return rc;
}
