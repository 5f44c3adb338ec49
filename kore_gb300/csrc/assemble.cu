// Assembly of a pencil's block-structured matrices on the GPU: what bin/assemble.py does
// with the radial operators (the .mtx submatrices) of bin/submatrices.py
// (bin/assemble.py:606-1176).
//
// The unknowns are blocks of n1 radial coefficients (one block per degree l and
// section).  Every nonzero block (R, C) of the matrix is a sum of radial operators scaled
// by coefficients that depend on the degree of block R: entries (R, C, op, coef), sorted
// by R.  The first g_R rows of block R hold its boundary rows instead (dense rows of n1
// values).  The caller gives, per row block, a pattern signature: for each local row
// i of the block, the (block offset dC, local column j) pairs of that row's entries
// (the union of the operators' row patterns), in increasing global column order.
// Row blocks that couple to the same offsets with the same operators share one.
//
// One warp per matrix row writes the row's column indices and values:
//   value(R, i; C, j) = bc_R[i][j]                          for i < g_R (C = R),
//                     = sum_e coef_e op_e[i][j] over entries e = (R, C, op_e, coef_e)   otherwise,
// with the operators read from dense n1 x n1 copies in device memory (tens of MB).
#include "kore_internal.cuh"

namespace {

struct AsmArgs {
    int n1;
    int64_t nrows;
    const double2 *ops;        // nops x n1 x n1, row-major
    const int *sig_of;         // row block -> signature
    const int *sig_rowptr;     // nsig x (n1 + 1)
    const int2 *sig_pat;       // (dC, j)
    const int64_t *ent_ptr;    // row block -> [begin, end) of its entries
    const int *ent_col;        // column block of the entry
    const int *ent_op;         // operator of the entry
    const double2 *ent_coef;   // coefficient of the entry
    const int *bc_g;           // boundary rows of the row block
    const int64_t *bc_ptr;     // offset of its boundary rows in bc_vals (g x n1, row-major)
    const double2 *bc_vals;
    const int64_t *indptr;     // nrows + 1
    int *indices;
    double2 *values;
};

__global__ void k_assemble(AsmArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t n1 = a.n1, SS = n1 * n1;
    for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < a.nrows; r += nw) {
        const int64_t R = r / n1;
        const int i = (int)(r - R * n1);
        const int sig = a.sig_of[R];
        const int p0 = a.sig_rowptr[(int64_t)sig * (n1 + 1) + i], p1 = a.sig_rowptr[(int64_t)sig * (n1 + 1) + i + 1];
        const int64_t out = a.indptr[r];
        const int g = a.bc_g[R];
        const int64_t e0 = a.ent_ptr[R], e1 = a.ent_ptr[R + 1];
        for (int p = p0 + lane; p < p1; p += 32) {
            const int2 pc = a.sig_pat[p];
            const int64_t C = R + pc.x;
            const int j = pc.y;
            double2 v = mk(0.0, 0.0);
            if (i < g) {
                if (pc.x == 0) v = a.bc_vals[a.bc_ptr[R] + (int64_t)i * n1 + j];
            } else {
                for (int64_t e = e0; e < e1; ++e)
                    if (a.ent_col[e] == C) v = v + a.ent_coef[e] * a.ops[a.ent_op[e] * SS + (int64_t)i * n1 + j];
            }
            a.indices[out + (p - p0)] = (int)(C * n1 + j);
            a.values[out + (p - p0)] = v;
        }
    }
}

}  // namespace

extern "C" int kore_assemble_blocks(int device, int n1, int nops, const double *ops, int64_t nrowblk,
                                    const int32_t *sig_of, int nsig, const int32_t *sig_rowptr, int64_t npat,
                                    const int32_t *sig_pat, const int64_t *ent_ptr, const int32_t *ent_col,
                                    const int32_t *ent_op, const double *ent_coef, const int32_t *bc_g,
                                    const int64_t *bc_ptr, int64_t bc_len, const double *bc_vals,
                                    const int64_t *indptr, int64_t nnz, int32_t *indices, double *values) {
    if (n1 <= 0 || nops <= 0 || !ops || nrowblk <= 0 || !sig_of || nsig <= 0 || !sig_rowptr || npat < 0 ||
        (npat > 0 && !sig_pat) || !ent_ptr || !ent_col || !ent_op || !ent_coef || !bc_g || !bc_ptr || bc_len < 0 ||
        (bc_len > 0 && !bc_vals) || !indptr || nnz < 0 || !indices || !values)
        return KORE_EINVAL;
    const int64_t nrows = nrowblk * n1;
    if (indptr[0] != 0 || indptr[nrows] != nnz || nnz > INT32_MAX || nrows > INT32_MAX) return KORE_EINVAL;
    // the arrays must describe each other: signatures, entries and boundary rows in range
    const int64_t nent = ent_ptr[nrowblk];
    if (ent_ptr[0] != 0) return KORE_EINVAL;
    for (int64_t R = 0; R < nrowblk; ++R) {
        if (sig_of[R] < 0 || sig_of[R] >= nsig || ent_ptr[R] > ent_ptr[R + 1] || bc_g[R] < 0 || bc_g[R] > n1)
            return KORE_EINVAL;
        if (bc_g[R] > 0 && (bc_ptr[R] < 0 || bc_ptr[R] + (int64_t)bc_g[R] * n1 > bc_len)) return KORE_EINVAL;
        const int s = sig_of[R];
        for (int i = 0; i < n1; ++i)
            if (indptr[R * n1 + i + 1] - indptr[R * n1 + i] != sig_rowptr[(int64_t)s * (n1 + 1) + i + 1] -
                                                                  sig_rowptr[(int64_t)s * (n1 + 1) + i])
                return KORE_EINVAL;
    }
    for (int64_t e = 0; e < nent; ++e)
        if (ent_op[e] < 0 || ent_op[e] >= nops || ent_col[e] < 0 || ent_col[e] >= nrowblk) return KORE_EINVAL;
    for (int64_t p = 0; p < npat; ++p) {
        if (sig_pat[2 * p + 1] < 0 || sig_pat[2 * p + 1] >= n1) return KORE_EINVAL;
    }
    for (int s = 0; s < nsig; ++s) {
        const int32_t *rp = sig_rowptr + (int64_t)s * (n1 + 1);
        if (rp[0] < 0 || rp[n1] > npat) return KORE_EINVAL;
        for (int i = 0; i < n1; ++i)
            if (rp[i + 1] < rp[i]) return KORE_EINVAL;
    }
    for (int64_t R = 0; R < nrowblk; ++R) {   // every column block of a pattern entry exists
        const int s = sig_of[R];
        for (int p = sig_rowptr[(int64_t)s * (n1 + 1)]; p < sig_rowptr[(int64_t)s * (n1 + 1) + n1]; ++p) {
            const int64_t C = R + sig_pat[2 * p];
            if (C < 0 || C >= nrowblk) return KORE_EINVAL;
        }
    }

    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device) KORE_CUDA_TRY(cudaSetDevice(device));
    int rc = KORE_OK;
    auto ck = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == KORE_OK) rc = (e == cudaErrorMemoryAllocation) ? KORE_ENOMEM : KORE_ECUDA;
    };
    const size_t ops_b = (size_t)nops * n1 * n1 * sizeof(double2);
    double2 *d_ops = nullptr, *d_coef = nullptr, *d_bc = nullptr, *d_val = nullptr;
    int *d_sig_of = nullptr, *d_sig_rowptr = nullptr, *d_ent_col = nullptr, *d_ent_op = nullptr, *d_bcg = nullptr,
        *d_idx = nullptr;
    int2 *d_pat = nullptr;
    int64_t *d_ent_ptr = nullptr, *d_bcp = nullptr, *d_indptr = nullptr;
    cudaStream_t st = nullptr;
    ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    ck(cudaMalloc(&d_ops, ops_b));
    ck(cudaMalloc(&d_sig_of, nrowblk * sizeof(int)));
    ck(cudaMalloc(&d_sig_rowptr, (size_t)nsig * (n1 + 1) * sizeof(int)));
    ck(cudaMalloc(&d_pat, std::max<int64_t>(npat, 1) * sizeof(int2)));
    ck(cudaMalloc(&d_ent_ptr, (nrowblk + 1) * sizeof(int64_t)));
    ck(cudaMalloc(&d_ent_col, std::max<int64_t>(nent, 1) * sizeof(int)));
    ck(cudaMalloc(&d_ent_op, std::max<int64_t>(nent, 1) * sizeof(int)));
    ck(cudaMalloc(&d_coef, std::max<int64_t>(nent, 1) * sizeof(double2)));
    ck(cudaMalloc(&d_bcg, nrowblk * sizeof(int)));
    ck(cudaMalloc(&d_bcp, nrowblk * sizeof(int64_t)));
    ck(cudaMalloc(&d_bc, std::max<int64_t>(bc_len, 1) * sizeof(double2)));
    ck(cudaMalloc(&d_indptr, (nrows + 1) * sizeof(int64_t)));
    ck(cudaMalloc(&d_idx, std::max<int64_t>(nnz, 1) * sizeof(int)));
    ck(cudaMalloc(&d_val, std::max<int64_t>(nnz, 1) * sizeof(double2)));
    if (rc == KORE_OK) {
        ck(cudaMemcpyAsync(d_ops, ops, ops_b, cudaMemcpyHostToDevice, st));
        ck(cudaMemcpyAsync(d_sig_of, sig_of, nrowblk * sizeof(int), cudaMemcpyHostToDevice, st));
        ck(cudaMemcpyAsync(d_sig_rowptr, sig_rowptr, (size_t)nsig * (n1 + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
        if (npat > 0) ck(cudaMemcpyAsync(d_pat, sig_pat, npat * sizeof(int2), cudaMemcpyHostToDevice, st));
        ck(cudaMemcpyAsync(d_ent_ptr, ent_ptr, (nrowblk + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        if (nent > 0) {
            ck(cudaMemcpyAsync(d_ent_col, ent_col, nent * sizeof(int), cudaMemcpyHostToDevice, st));
            ck(cudaMemcpyAsync(d_ent_op, ent_op, nent * sizeof(int), cudaMemcpyHostToDevice, st));
            ck(cudaMemcpyAsync(d_coef, ent_coef, nent * sizeof(double2), cudaMemcpyHostToDevice, st));
        }
        ck(cudaMemcpyAsync(d_bcg, bc_g, nrowblk * sizeof(int), cudaMemcpyHostToDevice, st));
        ck(cudaMemcpyAsync(d_bcp, bc_ptr, nrowblk * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        if (bc_len > 0) ck(cudaMemcpyAsync(d_bc, bc_vals, bc_len * sizeof(double2), cudaMemcpyHostToDevice, st));
        ck(cudaMemcpyAsync(d_indptr, indptr, (nrows + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        AsmArgs a{n1, nrows, d_ops, d_sig_of, d_sig_rowptr, d_pat, d_ent_ptr, d_ent_col, d_ent_op, d_coef,
                  d_bcg, d_bcp, d_bc, d_indptr, d_idx, d_val};
        int nsm = 0;
        ck(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
        const unsigned grid = (unsigned)std::min<int64_t>(kore_div_up(nrows * 32, 256), (int64_t)nsm * 16);
        k_assemble<<<std::max(1u, grid), 256, 0, st>>>(a);
        KORE_LAUNCHED(1);
        ck(cudaGetLastError());
        if (nnz > 0) {
            ck(cudaMemcpyAsync(indices, d_idx, nnz * sizeof(int), cudaMemcpyDeviceToHost, st));
            ck(cudaMemcpyAsync(values, d_val, nnz * sizeof(double2), cudaMemcpyDeviceToHost, st));
        }
        ck(cudaStreamSynchronize(st));
    }
    cudaFree(d_ops); cudaFree(d_sig_of); cudaFree(d_sig_rowptr); cudaFree(d_pat); cudaFree(d_ent_ptr);
    cudaFree(d_ent_col); cudaFree(d_ent_op); cudaFree(d_coef); cudaFree(d_bcg); cudaFree(d_bcp); cudaFree(d_bc);
    cudaFree(d_indptr); cudaFree(d_idx); cudaFree(d_val);
    if (st) cudaStreamDestroy(st);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return rc;
}
