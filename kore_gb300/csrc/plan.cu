// Plan creation and the extern "C" entry points of libkoregpu (include/kore_gpu.h).
//
// kore_plan_create replaces the matrix loading of bin/solve.py:40-86: it takes the
// CSR arrays that bin/assemble.py saved (np.savez, loaded by bin/utils.py:1253-1256),
// applies the l-major permutation, renumbers rows and columns into padded block
// slots (block i -> [i*S, (i+1)*S)), checks that every entry of A lies in the
// block-tridiagonal band and every entry of B in a diagonal block, and uploads the
// result.  The rows keep their entries sorted by column so each row splits into its
// L (block i-1), D (block i) and U (block i+1) segments.
#include "kore_internal.cuh"
#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <memory>
#include <cmath>
#include <vector>

std::atomic<long long> g_kore_launches{0};

int kore_alloc(kore_plan *p, void **ptr, size_t bytes) {
    *ptr = nullptr;
    if (bytes == 0) return KORE_OK;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return (e == cudaErrorMemoryAllocation) ? KORE_ENOMEM : KORE_ECUDA;
    }
    p->bytes += bytes;
    return KORE_OK;
}

int kore_check_device_error(kore_plan *p) {
    int h = 0;
    KORE_CUDA_TRY(cudaMemcpy(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h == 0) return KORE_OK;
    KORE_CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
    if (h == KORE_DEVERR_PIVOT) return KORE_ESINGULAR;
    return KORE_ETIMEOUT;
}

int kore_prof_mark(kore_plan *p, int kind, bool begin) {
    if (p->ev_used == p->ev_pool.size()) {
        cudaEvent_t e;
        KORE_CUDA_TRY(cudaEventCreate(&e));
        p->ev_pool.push_back(e);
    }
    const size_t idx = p->ev_used++;
    KORE_CUDA_TRY(cudaEventRecord(p->ev_pool[idx], p->stream));
    if (begin) p->ev_marks.push_back({kind, idx});
    return KORE_OK;
}

// Sum the elapsed times of all recorded (start, stop) pairs and recycle the events.
int kore_prof_collect(kore_plan *p) {
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    for (const auto &m : p->ev_marks) {
        if (m.second + 1 >= p->ev_used) continue;
        float ms = 0.f;
        KORE_CUDA_TRY(cudaEventElapsedTime(&ms, p->ev_pool[m.second], p->ev_pool[m.second + 1]));
        p->prof_ms[m.first] += ms;
        p->prof_n[m.first] += 1;
    }
    p->ev_marks.clear();
    p->ev_used = 0;
    return KORE_OK;
}

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

template <typename T>
int upload(kore_plan *p, T **dst, const std::vector<T> &src) {
    KORE_TRY(kore_alloc(p, (void **)dst, src.size() * sizeof(T)));
    if (!src.empty()) KORE_CUDA_TRY(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return KORE_OK;
}

void free_plan(kore_plan *p) {
    for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
    p->ev_pool.clear();
    void *ptrs[] = {p->d_arow, p->d_acol, p->d_asplit, p->d_aval, p->d_brow, p->d_bcol, p->d_bval,
                    p->d_slot2orig, p->d_bsz, p->d_Dinv, p->d_Gm, p->d_Hm, p->d_Dw, p->d_LU, p->d_lev,
                    p->d_rscale, p->d_T, p->d_piv, p->d_pidx, p->d_used, p->d_zlo, p->d_xlo, p->d_flo,
                    p->d_red, p->d_part, p->d_err, p->d_bar, p->d_ir, p->d_V, p->d_Vtmp, p->d_ksx, p->d_small, p->d_warm,
                    p->d_sigma, p->d_minf, p->d_bb, p->d_xb, p->d_rb, p->d_bn, p->d_rn, p->d_cnt,
                    p->d_ell_col, p->d_ell_src, p->d_ell_val, p->d_long_rows, p->d_srow, p->d_smid,
                    p->d_scol, p->d_sval, p->d_cc_ptr, p->d_cc_row, p->d_cc_src};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    for (auto &v : p->d_v)
        if (v) cudaFree(v);
    if (p->h_red) cudaFreeHost(p->h_red);
    if (p->stream) cudaStreamDestroy(p->stream);
}

// Permute one CSR matrix.  band = 1: blocks i-1..i+1 allowed (A); band = 0: block i only (B).
template <typename V>
int permute_csr(const kore_plan *p, const std::vector<int64_t> &orig2slot, const std::vector<int64_t> &slot2orig,
                const int32_t *indptr, const int32_t *indices, const V *data, int band, std::vector<int> &row,
                std::vector<int> &col, std::vector<V> &val, std::vector<int> *split) {
    const int64_t np = p->np, S = p->S;
    row.assign(np + 1, 0);
    for (int64_t s = 0; s < np; ++s) {
        const int64_t o = slot2orig[s];
        row[s + 1] = row[s] + (o >= 0 ? indptr[o + 1] - indptr[o] : 0);
    }
    const int64_t nnz = row[np];
    col.resize(nnz);
    val.resize(nnz);
    if (split) split->assign(2 * np, 0);
    int bad = 0;
#pragma omp parallel reduction(+ : bad)
    {
        std::vector<std::pair<int64_t, int>> tmp;   // one sort buffer per thread
#pragma omp for schedule(dynamic, 256)
        for (int64_t s = 0; s < np; ++s) {
            const int64_t o = slot2orig[s];
            const int64_t blk = s / S;
            const int b0 = row[s];
            if (o < 0) {
                if (split) { (*split)[2 * s] = b0; (*split)[2 * s + 1] = b0; }
                continue;
            }
            const int e0 = indptr[o], e1 = indptr[o + 1];
            tmp.resize(e1 - e0);
            for (int e = e0; e < e1; ++e) {
                const int64_t c = orig2slot[indices[e]];
                const int64_t cb = c / S;
                if (cb < blk - band || cb > blk + band) ++bad;
                tmp[e - e0] = {c, e};
            }
            std::sort(tmp.begin(), tmp.end());
            int d0 = -1, u0 = -1;
            for (size_t t = 0; t < tmp.size(); ++t) {
                col[b0 + t] = (int)tmp[t].first;
                val[b0 + t] = data[tmp[t].second];
                const int64_t cb = tmp[t].first / S;
                if (d0 < 0 && cb >= blk) d0 = b0 + (int)t;
                if (u0 < 0 && cb >= blk + 1) u0 = b0 + (int)t;
            }
            const int end = b0 + (int)tmp.size();
            if (d0 < 0) d0 = end;
            if (u0 < 0) u0 = end;
            if (split) { (*split)[2 * s] = d0; (*split)[2 * s + 1] = u0; }
        }
    }
    return bad ? KORE_EINVAL : KORE_OK;
}

// Padded coupling rows of the level-0 blocks (kore_plan::d_ell_*) from the
// permuted CSR of A: the entries left of the diagonal block, then those right of it.
int build_ell(kore_plan *p, const std::vector<int> &row, const std::vector<int> &col, const std::vector<int> &split) {
    const int64_t S = p->S;
    const int nt = (int)((S + 31) / 32);
    const int64_t nb = p->nlev > 0 ? p->K : 0;
    int w = 1;
#pragma omp parallel for reduction(max : w)
    for (int64_t q = 0; q < nb * S; ++q) w = std::max(w, (split[2 * q] - row[q]) + (row[q + 1] - split[2 * q + 1]));
    p->ell_w = (w + 7) & ~7;
    p->ell_rows = nb * nt * 32;
    std::vector<int> ecol(std::max<int64_t>(p->ell_stride(), 1), -1), esrc(ecol.size(), -1);
    int64_t ennz = 0;
#pragma omp parallel for reduction(+ : ennz)
    for (int64_t q = 0; q < nb * S; ++q) {
        const int64_t bi = q / S, r = q - bi * S;
        const int64_t base = ((bi * nt + r / 32) * p->ell_w) * 32 + r % 32;
        int k = 0;
        auto put = [&](int e) {
            ecol[base + (int64_t)k * 32] = col[e];
            esrc[base + (int64_t)k * 32] = e;
            ++k;
        };
        for (int e = row[q]; e < split[2 * q]; ++e) put(e);
        for (int e = split[2 * q + 1]; e < row[q + 1]; ++e) put(e);
        ennz += k;
    }
    p->ell_nnz = ennz;
    KORE_TRY(upload(p, &p->d_ell_col, ecol));
    KORE_TRY(upload(p, &p->d_ell_src, esrc));
    // The odd blocks' couplings by column (G_j = D_j^-1 L_j, H_j = D_j^-1 U_j at level 0):
    // task t = 2 o + side holds the entries of block j = 2 o + 1 in the columns of its
    // left (side 0) or right (side 1) neighbour, column by column, rows ascending.
    // Counted per column first, then filled, each task on its own thread.
    const int64_t no = p->nlev > 0 ? p->lev[0].nodd : 0, ntask = 2 * no;
    std::vector<int> cptr(std::max<int64_t>(ntask * (S + 1), 1), 0);
    auto entries = [&](int64_t t, int64_t r, int &e0, int &e1) {
        const int64_t j = 2 * (t / 2) + 1, q = j * S + r;
        e0 = (t & 1) ? split[2 * q + 1] : row[q];
        e1 = (t & 1) ? row[q + 1] : split[2 * q];
    };
    auto nbr_of = [&](int64_t t) -> int64_t { return (t & 1) ? 2 * (t / 2) + 2 : 2 * (t / 2); };
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t t = 0; t < ntask; ++t) {
        int *cnt = &cptr[t * (S + 1)];
        for (int64_t r = 0; r < S; ++r) {
            int e0, e1;
            entries(t, r, e0, e1);
            for (int e = e0; e < e1; ++e) ++cnt[col[e] - nbr_of(t) * S + 1];
        }
    }
    // offsets: each task's columns follow the previous task's
    int64_t total = 0;
    for (int64_t t = 0; t < ntask; ++t) {
        int *ptr = &cptr[t * (S + 1)];
        ptr[0] = (int)total;
        for (int64_t c = 0; c < S; ++c) ptr[c + 1] += ptr[c];
        total = ptr[S];
    }
    std::vector<int> crow(std::max<int64_t>(total, 1), 0), csrc(crow.size(), 0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t t = 0; t < ntask; ++t) {
        const int *ptr = &cptr[t * (S + 1)];
        std::vector<int> cur(ptr, ptr + S);
        for (int64_t r = 0; r < S; ++r) {
            int e0, e1;
            entries(t, r, e0, e1);
            for (int e = e0; e < e1; ++e) {
                const int k = cur[col[e] - nbr_of(t) * S]++;
                crow[k] = (int)r;
                csrc[k] = e;
            }
        }
    }
    KORE_TRY(upload(p, &p->d_cc_ptr, cptr));
    KORE_TRY(upload(p, &p->d_cc_row, crow));
    KORE_TRY(upload(p, &p->d_cc_src, csrc));
    return KORE_OK;
}

int create(const kore_pencil_desc *d, int device, kore_plan **out) {
    if (!d || !out || d->n <= 0 || d->nblocks <= 0 || !d->block_sizes || !d->perm || !d->a_indptr)
        return KORE_EINVAL;
    if (d->a_nnz >= (int64_t)INT32_MAX || d->b_nnz >= (int64_t)INT32_MAX) return KORE_EINVAL;
    DeviceGuard g(device);
    auto *p = new kore_plan();
    std::unique_ptr<kore_plan, void (*)(kore_plan *)> guard(p, [](kore_plan *q) { free_plan(q); delete q; });
    p->device = device;
    p->n = d->n;
    p->K = d->nblocks;
    p->bsz.assign(d->block_sizes, d->block_sizes + d->nblocks);
    p->boff.resize(p->K + 1, 0);
    for (int i = 0; i < p->K; ++i) {
        if (p->bsz[i] <= 0) return KORE_EINVAL;
        p->boff[i + 1] = p->boff[i] + p->bsz[i];
    }
    if (p->boff[p->K] != p->n) return KORE_EINVAL;
    // padded block size: a multiple of 4 so that every factor column (S complex64
    // entries) starts on a 32-byte boundary, as the tensor-copy sweep needs
    p->S = (*std::max_element(p->bsz.begin(), p->bsz.end()) + 3) & ~3;
    if (p->S > 1024) return KORE_EINVAL;
    p->np = (int64_t)p->K * p->S;
    if (p->np * 8 >= (int64_t)INT32_MAX) return KORE_EINVAL;

    std::vector<int64_t> orig2slot(p->n, -1), slot2orig(p->np, -1);
    for (int i = 0; i < p->K; ++i)
        for (int k = 0; k < p->bsz[i]; ++k) {
            const int64_t q = p->boff[i] + k;
            const int64_t o = d->perm[q];
            if (o < 0 || o >= p->n || orig2slot[o] >= 0) return KORE_EINVAL;
            orig2slot[o] = (int64_t)i * p->S + k;
            slot2orig[(int64_t)i * p->S + k] = o;
        }

    kore_build_levels(p);
    KORE_CUDA_TRY(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    KORE_CUDA_TRY(cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, device));
    KORE_TRY(kore_spmv_prepare(p));

    std::vector<int> rowlen;
    {
        std::vector<int> row, col, split;
        std::vector<double2> val;
        const double2 *adata = reinterpret_cast<const double2 *>(d->a_data);
        KORE_TRY(permute_csr(p, orig2slot, slot2orig, d->a_indptr, d->a_indices, adata, 1, row, col, val, &split));
        p->a_nnz = (int64_t)col.size();
        KORE_TRY(upload(p, &p->d_arow, row));
        KORE_TRY(upload(p, &p->d_acol, col));
        KORE_TRY(upload(p, &p->d_aval, val));
        KORE_TRY(upload(p, &p->d_asplit, split));
        KORE_TRY(build_ell(p, row, col, split));
        // real/imaginary split of A for the sparse products: per row the values with a
        // nonzero real part, then those with a nonzero imaginary part (counted, then
        // filled, rows in parallel)
        std::vector<int> srow(p->np + 1, 0), smid(p->np), nre(p->np), nim(p->np);
#pragma omp parallel for schedule(static, 1024)
        for (int64_t q = 0; q < p->np; ++q) {
            int a = 0, b = 0;
            for (int e = row[q]; e < row[q + 1]; ++e) {
                a += val[e].x != 0.0;
                b += val[e].y != 0.0;
            }
            nre[q] = a;
            nim[q] = b;
        }
        int64_t stot = 0;
        for (int64_t q = 0; q < p->np; ++q) {
            if (stot + nre[q] + nim[q] >= (int64_t)INT32_MAX) return KORE_EINVAL;
            smid[q] = (int)(stot + nre[q]);
            stot += nre[q] + nim[q];
            srow[q + 1] = (int)stot;
        }
        std::vector<int> scol(std::max<int64_t>(stot, 1));
        std::vector<double> sval(scol.size());
#pragma omp parallel for schedule(static, 1024)
        for (int64_t q = 0; q < p->np; ++q) {
            int kr = srow[q], ki = smid[q];
            for (int e = row[q]; e < row[q + 1]; ++e) {
                if (val[e].x != 0.0) { scol[kr] = col[e]; sval[kr] = val[e].x; ++kr; }
                if (val[e].y != 0.0) { scol[ki] = col[e]; sval[ki] = val[e].y; ++ki; }
            }
        }
        p->s_nnz = stot;
        KORE_TRY(upload(p, &p->d_srow, srow));
        KORE_TRY(upload(p, &p->d_smid, smid));
        KORE_TRY(upload(p, &p->d_scol, scol));
        KORE_TRY(upload(p, &p->d_sval, sval));
        rowlen.resize(p->np);
        for (int64_t q = 0; q < p->np; ++q) rowlen[q] = srow[q + 1] - srow[q];
    }
    p->has_b = d->b_nnz > 0 && d->b_indptr && d->b_indices && d->b_data;
    if (p->has_b) {
        std::vector<int> row, col;
        std::vector<double> val;
        KORE_TRY(permute_csr(p, orig2slot, slot2orig, d->b_indptr, d->b_indices, d->b_data, 0, row, col, val, nullptr));
        p->b_nnz = (int64_t)col.size();
        KORE_TRY(upload(p, &p->d_brow, row));
        KORE_TRY(upload(p, &p->d_bcol, col));
        KORE_TRY(upload(p, &p->d_bval, val));
        for (int64_t q = 0; q < p->np; ++q) rowlen[q] += row[q + 1] - row[q];
    }
    {
        // rows with more than kKoreLongRow stored values (the sparse products give them a warp each)
        std::vector<int> longr;
        for (int64_t q = 0; q < p->np; ++q)
            if (rowlen[q] > kKoreLongRow) longr.push_back((int)q);
        p->nlong = (int)longr.size();
        if (longr.empty()) longr.push_back(0);
        KORE_TRY(upload(p, &p->d_long_rows, longr));
    }
    KORE_TRY(upload(p, &p->d_slot2orig, slot2orig));
    KORE_TRY(upload(p, &p->d_bsz, p->bsz));
    if (!p->lev.empty()) {
        KORE_TRY(kore_alloc(p, (void **)&p->d_lev, p->lev.size() * sizeof(BcrLevel)));
        KORE_CUDA_TRY(cudaMemcpy(p->d_lev, p->lev.data(), p->lev.size() * sizeof(BcrLevel), cudaMemcpyHostToDevice));
    }
    for (auto &v : p->d_v) KORE_TRY(kore_alloc(p, (void **)&v, p->np * sizeof(double2)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_red, 8192 * sizeof(double)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_err, sizeof(int)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_bar, 64));
    KORE_CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
    KORE_CUDA_TRY(cudaMemset(p->d_red, 0, 8192 * sizeof(double)));
    KORE_CUDA_TRY(cudaMallocHost(&p->h_red, 8192 * sizeof(double)));
    // the set-up copies and memsets ran on the legacy default stream; plans' own streams
    // are non-blocking, so this waits for this plan's set-up only
    KORE_CUDA_TRY(cudaStreamSynchronize(0));
    *out = guard.release();
    return KORE_OK;
}

// nrhs right-hand sides (original order, device) in groups of nshift: right-hand side k
// is solved with shift k % nshift.
int solve_dev_impl(kore_plan *p, const double2 *b, double2 *x, int nrhs, double tol, kore_stats *st) {
    if (nrhs % p->nshift != 0) return KORE_EINVAL;
    KORE_TRY(kore_ir_reset(p));
    for (int g = 0; g < nrhs; g += p->nshift) {
        KORE_TRY(kore_gather_shifts(p, b + (int64_t)g * p->n, p->d_bb));
        KORE_TRY(kore_apply_inverse(p, p->d_bb, p->d_xb, tol));
        KORE_TRY(kore_scatter_shifts(p, p->d_xb, x + (int64_t)g * p->n));
    }
    IrState s;
    KORE_TRY(kore_ir_read(p, &s));
    if (st) {
        st->sweeps = s.sweeps;
        st->refine_iters_max = s.iters_max;
        st->solve_resid_max = s.eta_max;
    }
    if (s.nan) return KORE_ENAN;
    return KORE_OK;
}

}  // namespace

extern "C" {

int kore_plan_create(const kore_pencil_desc *desc, int device, kore_plan **plan) {
    if (plan) *plan = nullptr;
    return create(desc, device, plan);
}

int kore_factor(kore_plan *plan, double sigma_re, double sigma_im, int precision) {
    if (!plan) return KORE_EINVAL;
    DeviceGuard g(plan->device);
    const double sig[2] = {sigma_re, sigma_im};
    return kore_factor_impl(plan, 1, sig, precision);
}

int kore_factor_shifts(kore_plan *plan, int nshift, const double *sigmas, int precision) {
    if (!plan || nshift <= 0 || !sigmas) return KORE_EINVAL;
    DeviceGuard g(plan->device);
    return kore_factor_impl(plan, nshift, sigmas, precision);
}

int kore_solve(kore_plan *p, const double *b, double *x, int nrhs, double refine_tol, kore_stats *stats) {
    if (!p || !b || !x || nrhs <= 0) return KORE_EINVAL;
    if (p->factored && nrhs % p->nshift != 0) return KORE_EINVAL;
    if (!p->factored) return KORE_ENOTFACTORED;
    DeviceGuard g(p->device);
    auto t0 = std::chrono::steady_clock::now();
    if (stats) *stats = kore_stats{};
    double2 *db = nullptr, *dx = nullptr;
    const size_t bytes = (size_t)p->n * nrhs * sizeof(double2);
    KORE_CUDA_TRY(cudaMallocAsync((void **)&db, bytes, p->stream));
    KORE_CUDA_TRY(cudaMallocAsync((void **)&dx, bytes, p->stream));
    int s = KORE_OK;
    if (cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, p->stream) != cudaSuccess) s = KORE_ECUDA;
    if (s == KORE_OK) s = solve_dev_impl(p, db, dx, nrhs, refine_tol, stats);
    if (s == KORE_OK && cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess) s = KORE_ECUDA;
    cudaFreeAsync(db, p->stream);
    cudaFreeAsync(dx, p->stream);
    if (cudaStreamSynchronize(p->stream) != cudaSuccess && s == KORE_OK) s = KORE_ECUDA;
    if (s == KORE_OK) s = kore_check_device_error(p);
    if (s == KORE_OK)
        for (int64_t i = 0; i < 2 * p->n * nrhs; ++i)
            if (!std::isfinite(x[i])) { s = KORE_ENAN; break; }
    if (stats) stats->iterate_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return s;
}

int kore_solve_dev(kore_plan *p, const void *b_dev, void *x_dev, int nrhs, double refine_tol, void *stream,
                   kore_stats *stats) {
    if (!p || !b_dev || !x_dev || nrhs <= 0) return KORE_EINVAL;
    if (!p->factored) return KORE_ENOTFACTORED;
    DeviceGuard g(p->device);
    if (stats) *stats = kore_stats{};
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    cudaEvent_t ev;
    KORE_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    KORE_CUDA_TRY(cudaEventRecord(ev, cs));
    KORE_CUDA_TRY(cudaStreamWaitEvent(p->stream, ev, 0));
    int s = solve_dev_impl(p, static_cast<const double2 *>(b_dev), static_cast<double2 *>(x_dev), nrhs, refine_tol, stats);
    KORE_CUDA_TRY(cudaEventRecord(ev, p->stream));
    KORE_CUDA_TRY(cudaStreamWaitEvent(cs, ev, 0));
    cudaEventDestroy(ev);
    if (s == KORE_OK) s = kore_check_device_error(p);
    return s;
}

int kore_eigs(kore_plan *p, const kore_eps_opts *opts, double *evals, double *evecs, int max_pairs, int *nconv,
              kore_stats *stats) {
    if (!p || !opts || !evals || !nconv || max_pairs <= 0) return KORE_EINVAL;
    if (p->factored && p->nshift != 1) return KORE_EINVAL;
    DeviceGuard g(p->device);
    *nconv = 0;
    return kore_eigs_impl(p, 1, opts, evals, evecs, max_pairs, nconv, stats);
}

int kore_eigs_shifts(kore_plan *p, int ntarget, const kore_eps_opts *opts, double *evals, double *evecs,
                     int max_pairs, int *nconv, kore_stats *stats) {
    if (!p || ntarget <= 0 || !opts || !evals || !nconv || max_pairs <= 0) return KORE_EINVAL;
    if (p->factored && ntarget < p->nshift) return KORE_EINVAL;
    DeviceGuard g(p->device);
    for (int t = 0; t < ntarget; ++t) nconv[t] = 0;
    return kore_eigs_impl(p, ntarget, opts, evals, evecs, max_pairs, nconv, stats);
}

int kore_residual(kore_plan *p, double lre, double lim, const double *x, double *y) {
    if (!p || !x || !y) return KORE_EINVAL;
    DeviceGuard g(p->device);
    const size_t bytes = (size_t)p->n * sizeof(double2);
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_v[4], x, bytes, cudaMemcpyHostToDevice, p->stream));
    KORE_TRY(kore_gather(p, p->d_v[4], p->d_v[0]));
    KORE_TRY(kore_spmv_pencil(p, lre, lim, p->d_v[0], p->d_v[1]));
    KORE_TRY(kore_scatter(p, p->d_v[1], p->d_v[4]));
    KORE_CUDA_TRY(cudaMemcpyAsync(y, p->d_v[4], bytes, cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return KORE_OK;
}

int kore_plan_stream(const kore_plan *p, void **stream) {
    if (!p || !stream) return KORE_EINVAL;
    *stream = (void *)p->stream;
    return KORE_OK;
}

int kore_profile(kore_plan *p, int enable, double *out) {
    if (!p) return KORE_EINVAL;
    DeviceGuard g(p->device);
    KORE_TRY(kore_prof_collect(p));
    IrState irs{};
    if (p->d_ir) KORE_TRY(kore_ir_read(p, &irs));
    if (out) {
        const double e = p->factor_elt ? (double)p->factor_elt : 16.0;
        const double S = p->S, K = p->K, np = (double)p->np;
        out[0] = p->prof_ms[0];
        // sweeps that ran (sweep launches that returned at once, after the refinement
        // converged, are excluded: their events enclose no work)
        out[1] = (double)(irs.sweeps_total - p->sweeps_at_enable);
        out[2] = p->prof_ms[1];
        out[3] = (double)p->prof_n[1];
        // one sweep reads the D^-1, G, H blocks of the odd blocks of levels >= 1 and the
        // top block once, D^-1 of the level-0 odd blocks twice (no G, H at level 0), the
        // dense couplings of the even blocks of levels >= 1, the level-0 coupling rows of
        // every block (a value in factor precision + a 4 B index per entry), the
        // right-hand side (16 B) and row scales (8 B) and writes x (16 B); the reduction
        // vectors f, z, x in factor precision are read and written about twice each
        double lu = 0.0, mats = 1.0;
        for (int l = 0; l < p->nlev; ++l) {
            mats += (l == 0 ? 2.0 : 3.0) * p->lev[l].nodd;
            if (l > 0) lu += 2.0 * p->lev[l].neven;
        }
        out[4] = (mats + lu) * S * S * e + (double)p->ell_nnz * (e + 4.0) + np * (16.0 + 8.0 + 16.0) +
                 6.0 * np * e;
        // Gauss-Jordan on [D_j | L_j | U_j | I] for every eliminated block (trailing update
        // 8 S nb (4S - k0 - nb) real flops per panel, ~28 S^3 per block) and four dense
        // S^3 complex products (8 S^3 real flops each) per surviving block of levels >= 1
        double gj = 0.0, gm = 0.0;
        for (int l = 0; l < p->nlev; ++l) {
            gj += p->lev[l].nodd;
            if (l > 0) gm += 4.0 * p->lev[l].neven;
        }
        out[5] = (gj + 1.0) * 28.0 * S * S * S + gm * 8.0 * S * S * S;
        for (int k = 2; k < 5; ++k) {
            out[6 + 2 * (k - 2)] = p->prof_ms[k];
            out[7 + 2 * (k - 2)] = (double)p->prof_n[k];
        }
        out[12] = (double)p->sweep_cps;   // CTAs per SM of the last sweep (the autotuner's choice)
        out[13] = (double)p->sweep_chunk;   // and its ring chunk bytes
    }
    if (enable) {
        for (int k = 0; k < 5; ++k) { p->prof_ms[k] = 0.0; p->prof_n[k] = 0; }
        p->sweeps_at_enable = irs.sweeps_total;
    }
    p->prof = enable != 0;
    return KORE_OK;
}

int kore_plan_bytes(const kore_plan *p, int64_t *bytes) {
    if (!p || !bytes) return KORE_EINVAL;
    *bytes = (int64_t)p->bytes;
    return KORE_OK;
}

int64_t kore_kernel_launches(void) { return g_kore_launches.load(); }

int kore_plan_estimate_bytes(const kore_pencil_desc *d, int precision, int nshift, int ncv, int64_t *bytes) {
    if (!d || !bytes || d->n <= 0 || d->nblocks <= 0 || !d->block_sizes || !d->a_indptr || nshift <= 0) return KORE_EINVAL;
    if (precision != KORE_PREC_FP64 && precision != KORE_PREC_MIXED) return KORE_EINVAL;
    // the sizes the plan and ensure_factor_storage allocate (see create() and factor.cu)
    const int64_t K = d->nblocks;
    int64_t S = 0;
    for (int64_t i = 0; i < K; ++i) S = std::max<int64_t>(S, d->block_sizes[i]);
    S = (S + 3) & ~3LL;
    const int64_t np = K * S, SS = S * S, na = d->a_nnz, nb = d->b_nnz;
    std::vector<int64_t> Ks;
    for (int64_t Kl = K; Kl > 1; Kl -= Kl / 2) Ks.push_back(Kl);
    const int64_t nlev = (int64_t)Ks.size();
    int64_t lu = 0, nodd_max = 1;
    for (int64_t l = 0; l < nlev; ++l) {
        if (l > 0) lu += 2 * Ks[l];
        nodd_max = std::max<int64_t>(nodd_max, Ks[l] / 2);
    }
    lu = std::max<int64_t>(lu, 1);
    int64_t maxrow = 1;
    for (int64_t r = 0; r < d->n; ++r) maxrow = std::max<int64_t>(maxrow, d->a_indptr[r + 1] - d->a_indptr[r]);
    const int64_t nt = (S + 31) / 32;
    const int64_t ell = std::max<int64_t>((nlev > 0 ? K : 0) * nt * 32 * ((maxrow + 7) & ~7LL), 1);
    const int64_t e = (precision == KORE_PREC_FP64) ? 16 : 8, c = nshift;
    int64_t b = 0;
    // plan: A (CSR, split rows, padded level-0 rows), B, permutation, vectors
    b += (np + 1) * 4 + na * 20 + 2 * np * 4;
    b += (2 * np + 1) * 4 + 2 * na * 12;
    b += 2 * ell * 4 + np * 4;
    b += (np + 1) * 4 + nb * 12;
    b += np * 8 + K * 4 + nlev * (int64_t)sizeof(BcrLevel) + 6 * np * 16 + 8192 * 8 + 1024;
    // factors and solve workspace of c shifts
    b += c * (4 * K * SS * e + lu * SS * e + nodd_max * 2 * SS * e + 3 * np * e + np * 8 + 3 * nodd_max * S * 4);
    // level-0 couplings by column; split planes and job table of the tensor-core updates
    b += (2 * (K / 2 + 1) * (S + 1) + 2 * na) * 4;
    if (precision == KORE_PREC_MIXED) {
        const int64_t Kp = (S + 31) / 32 * 32;
        int64_t nm = 0, nj = 0;
        for (int64_t l = 0; l < nlev; ++l) {
            const int64_t ne = Ks[l] - Ks[l] / 2, no = Ks[l] / 2;
            nm = std::max<int64_t>(nm, std::max<int64_t>(l > 0 ? 4 * ne + 6 * no : 0, 4 * no + 6 * no) * 2);
            nj = std::max<int64_t>(nj, std::max<int64_t>(l > 0 ? 3 * ne : 0, 2 * no));
        }
        b += c * (nm / 2 * S * Kp * 4 + nm * 8 + nj * 32 + 64);   // nm / 2 planes of S x Kp floats
    }
    b += c * (3 * np * 16 + 2 * (np / 64 + np / 8 + 1024) * 8 + (nlev > 0 ? 3 * nlev + 2 : 1) * K * 4 + ell * e + 128);
    b += 2 * d->n * c * 16;   // kore_solve's device copies of b and x
    // per target (one per shift): Krylov basis, its restart copy, a gathered input vector,
    // the slot's warm-start vector and the projected-problem workspace
    if (ncv > 0) b += c * (2 * np * (int64_t)(ncv + 1) * 16 + 2 * np * 16 + (int64_t)(65 * 64 * 4 + 8 * 65 + 2048 * 65 + 4096) * 16);
    b += 128LL << 20;   // allocation granularity of ~50 buffers
    *bytes = b;
    return KORE_OK;
}

const char *kore_status_string(int s) {
    switch (s) {
        case KORE_OK: return "ok";
        case KORE_EINVAL: return "invalid argument or matrix outside the block-tridiagonal band";
        case KORE_ENOMEM: return "device allocation failed";
        case KORE_ECUDA: return "CUDA runtime error";
        case KORE_ESINGULAR: return "zero pivot in a diagonal Schur complement";
        case KORE_ENOCONV: return "no eigenpair converged";
        case KORE_ETIMEOUT: return "a bounded device wait ran out";
        case KORE_ENOTFACTORED: return "plan not factorised";
        case KORE_ENAN: return "NaN or Inf in the solution";
        case KORE_EPENDING: return "the request has not finished";
        case KORE_ECANCELLED: return "the request was cancelled before it started";
    }
    return "unknown status";
}

int kore_plan_destroy(kore_plan *p) {
    if (!p) return KORE_OK;
    DeviceGuard g(p->device);
    cudaStreamSynchronize(p->stream);
    free_plan(p);
    delete p;
    return KORE_OK;
}

}  // extern "C"
