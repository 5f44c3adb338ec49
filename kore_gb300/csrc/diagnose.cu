// Flow diagnostics of eigenvectors on the GPU: what bin/spin_doctor.py computes with
// bin/utils4pp.py (diagnose, flow_worker) for the hydrodynamic problem in a shell.
//
// For every degree l of a velocity eigenvector (poloidal coefficients P_l, toroidal
// T_l, N Chebyshev coefficients each, radius mapped to [ricb, rcmb]):
//   * the radial function and its r-derivatives at the N Chebyshev-Gauss points
//     x_i = cos((i + 1/2) pi / N) (bin/utils4pp.py:805-829, funcheb :28-51);
//   * the radial, consoidal and toroidal components q, s, t (cheb2space_pol/tor,
//     :163-218) and the integrands of the kinetic energy, of integral(u . lap u) and of
//     the internal dissipation (:221-296);
//   * their Chebyshev-Gauss quadratures (cg_quad, :54-64).
// The sums over l, the scaling by OmgTau Ek and the power-balance residuals
// (bin/spin_doctor.py:148-160, 225-236) are left to the caller (kore_gb300/diagnostics.py).
//
// Layout: k_cheb_eval writes E[j][i][k] = d^j T_k / dr^j (x_i) for j = 0..3 (one thread
// per point, three-term recurrences of T_k and its x-derivatives); k_flow_integrals
// runs one CTA per (degree block, eigenvector), the block's coefficients in shared
// memory, threads over the points, and reduces the three integrals in a fixed order.
#include "kore_internal.cuh"
#include <vector>

namespace {

constexpr int kDiagThreads = 256;

__global__ void k_cheb_eval(int N, double ricb, double rcmb, double *__restrict__ E) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double x = cos((i + 0.5) * 3.14159265358979323846 / N);
    const double dr = 2.0 / (rcmb - ricb);   // dx/dr
    const int64_t NN = (int64_t)N * N;
    // T_k and its first three x-derivatives: T_{k+1} = 2x T_k - T_{k-1} differentiated
    double t0 = 1.0, t1 = x;            // T_{k-1}, T_k
    double d10 = 0.0, d11 = 1.0;        // T'
    double d20 = 0.0, d21 = 0.0;        // T''
    double d30 = 0.0, d31 = 0.0;        // T'''
    for (int k = 0; k < N; ++k) {
        double v0, v1, v2, v3;
        if (k == 0) { v0 = 1.0; v1 = 0.0; v2 = 0.0; v3 = 0.0; }
        else if (k == 1) { v0 = x; v1 = 1.0; v2 = 0.0; v3 = 0.0; }
        else {
            const double n0 = 2.0 * x * t1 - t0;
            const double n1 = 2.0 * t1 + 2.0 * x * d11 - d10;
            const double n2 = 4.0 * d11 + 2.0 * x * d21 - d20;
            const double n3 = 6.0 * d21 + 2.0 * x * d31 - d30;
            t0 = t1; t1 = n0; d10 = d11; d11 = n1; d20 = d21; d21 = n2; d30 = d31; d31 = n3;
            v0 = n0; v1 = n1; v2 = n2; v3 = n3;
        }
        E[(int64_t)i * N + k] = v0;
        E[NN + (int64_t)i * N + k] = v1 * dr;
        E[2 * NN + (int64_t)i * N + k] = v2 * dr * dr;
        E[3 * NN + (int64_t)i * N + k] = v3 * dr * dr * dr;
    }
}

struct FlowArgs {
    int N, npol, ntor;
    double ricb, rcmb;
    const int *lpol, *ltor;      // degrees of the poloidal and toroidal blocks
    const double2 *x;            // nvec vectors of (npol + ntor) N complex coefficients
    const double *E;             // 4 N N evaluation matrices
    double *out;                 // per (vector, block): energy, diffusion, internal dissipation
};

__global__ void __launch_bounds__(kDiagThreads) k_flow_integrals(FlowArgs a) {
    extern __shared__ double2 cs[];   // the block's N coefficients
    __shared__ double red[3][kDiagThreads / 32];
    const int b = blockIdx.x, v = blockIdx.y, N = a.N;
    const int nblk = a.npol + a.ntor;
    const bool tor = b >= a.npol;
    const int l = tor ? a.ltor[b - a.npol] : a.lpol[b];
    const double2 *c = a.x + ((int64_t)v * nblk + b) * N;
    for (int k = threadIdx.x; k < N; k += blockDim.x) cs[k] = c[k];
    __syncthreads();
    const int64_t NN = (int64_t)N * N;
    const double L = (double)l * (l + 1), f0 = 4.0 * 3.14159265358979323846 / (2 * l + 1);
    double ke = 0.0, dk = 0.0, di = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double xk = cos((i + 0.5) * 3.14159265358979323846 / N);
        const double rk = 0.5 * (a.rcmb - a.ricb) * (xk + 1.0) + a.ricb;
        const double w = sqrt(1.0 - xk * xk);
        const int nd = tor ? 3 : 4;
        double2 p[4] = {mk(0, 0), mk(0, 0), mk(0, 0), mk(0, 0)};
        for (int j = 0; j < nd; ++j) {
            const double *e = a.E + j * NN + (int64_t)i * N;
            double2 acc = mk(0.0, 0.0);
            for (int k = 0; k < N; ++k) {
                const double ev = __ldg(e + k);
                acc.x = fma(ev, cs[k].x, acc.x);
                acc.y = fma(ev, cs[k].y, acc.y);
            }
            p[j] = acc;
        }
        const double r2 = rk * rk;
        double fke, fdk, fdi;
        if (!tor) {
            const double2 q0 = (L / rk) * p[0];
            const double2 s0 = p[1] + (1.0 / rk) * p[0];
            const double2 q1 = (1.0 / rk) * (L * p[1] - q0);
            const double2 s1 = p[2] + (1.0 / L) * q1;
            const double2 q2 = (1.0 / rk) * (L * p[2] - 2.0 * q1);
            const double2 s2 = p[3] + (1.0 / L) * q2;
            fke = f0 * (r2 * abs2(q0) + r2 * L * abs2(s0));
            const double2 t = L * r2 * (conjg(s0) * s2) + (2.0 * rk * L) * (conjg(s0) * s1) +
                              (-(L * L)) * (conjg(s0) * s0) + (-((double)l * l + l + 2)) * (conjg(q0) * q0) +
                              (2.0 * rk) * (conjg(q0) * q1) + r2 * (conjg(q0) * q2) +
                              (2.0 * L) * (conjg(q0) * s0 + q0 * conjg(s0));
            fdk = 2.0 * f0 * t.x;
            const double2 u = q0 + rk * s1 - s0;
            fdi = 2.0 * f0 * (L * abs2(u) + 3.0 * abs2(rk * q1) + L * (l - 1) * (l + 2) * abs2(s0));
        } else {
            const double2 t0 = p[0], t1 = p[1], t2 = p[2];
            fke = f0 * r2 * L * abs2(t0);
            const double2 t = L * r2 * (conjg(t0) * t2) + (2.0 * rk * L) * (conjg(t0) * t1) + (-(L * L)) * (conjg(t0) * t0);
            fdk = 2.0 * f0 * t.x;
            fdi = 2.0 * f0 * (L * abs2(rk * t1 - t0) + L * (l - 1) * (l + 2) * abs2(t0));
        }
        ke += w * fke;
        dk += w * fdk;
        di += w * fdi;
    }
    ke = warp_sum_d(ke);
    dk = warp_sum_d(dk);
    di = warp_sum_d(di);
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = ke;
        red[1][threadIdx.x >> 5] = dk;
        red[2][threadIdx.x >> 5] = di;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
        const double quad = (3.14159265358979323846 / N) * (a.rcmb - a.ricb) / 2.0;
        a.out[((int64_t)v * nblk + b) * 3 + threadIdx.x] = quad * s;
    }
}

}  // namespace

extern "C" int kore_flow_diagnostics(int device, int N, double ricb, int npol, const int32_t *lpol, int ntor,
                                     const int32_t *ltor, const double *x, int nvec, double *out) {
    if (N < 2 || N > 3000 || !(ricb > 0.0 && ricb < 1.0) || npol < 0 || ntor < 0 || npol + ntor == 0 ||
        (npol && !lpol) || (ntor && !ltor) || !x || nvec <= 0 || !out)
        return KORE_EINVAL;
    for (int b = 0; b < npol; ++b) if (lpol[b] < 1) return KORE_EINVAL;
    for (int b = 0; b < ntor; ++b) if (ltor[b] < 1) return KORE_EINVAL;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device) KORE_CUDA_TRY(cudaSetDevice(device));
    const int nblk = npol + ntor;
    const size_t xbytes = (size_t)nvec * nblk * N * sizeof(double2);
    const size_t obytes = (size_t)nvec * nblk * 3 * sizeof(double);
    double *dE = nullptr, *dout = nullptr;
    double2 *dx = nullptr;
    int *dl = nullptr;
    int rc = KORE_OK;
    auto ck = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == KORE_OK) rc = (e == cudaErrorMemoryAllocation) ? KORE_ENOMEM : KORE_ECUDA;
    };
    ck(cudaMalloc(&dE, (size_t)4 * N * N * sizeof(double)));
    ck(cudaMalloc(&dx, xbytes));
    ck(cudaMalloc(&dout, obytes));
    ck(cudaMalloc(&dl, (size_t)nblk * sizeof(int)));
    if (rc == KORE_OK) {
        std::vector<int> ls(lpol, lpol + npol);
        ls.insert(ls.end(), ltor, ltor + ntor);
        ck(cudaMemcpy(dl, ls.data(), ls.size() * sizeof(int), cudaMemcpyHostToDevice));
        ck(cudaMemcpy(dx, x, xbytes, cudaMemcpyHostToDevice));
        k_cheb_eval<<<kore_div_up(N, 128), 128>>>(N, ricb, 1.0, dE);
        FlowArgs a{N, npol, ntor, ricb, 1.0, dl, dl + npol, dx, dE, dout};
        k_flow_integrals<<<dim3(nblk, nvec), kDiagThreads, N * sizeof(double2)>>>(a);
        KORE_LAUNCHED(2);
        ck(cudaGetLastError());
        ck(cudaMemcpy(out, dout, obytes, cudaMemcpyDeviceToHost));
    }
    cudaFree(dE); cudaFree(dx); cudaFree(dout); cudaFree(dl);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return rc;
}
