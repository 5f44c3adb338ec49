// Complex64 GEMMs of the mixed-precision factorisation on the 5th-generation tensor
// cores (tcgen05), in three-pass TF32 (3xTF32):
//     x = x_hi + x_lo,  x_hi = x rounded to TF32,  x_lo = x - x_hi (exact in FP32),
//     a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi      (FP32 accumulation in tensor memory)
// and each complex product as four real ones,
//     Re(AB) = Ar Br - Ai Bi,  Im(AB) = Ar Bi + Ai Br,
// the subtraction done by the -Im planes of the B operand (below), so every MMA adds.
//
// Data flow of one 128 x 64 tile of C = beta C + alpha (A1 B1 [+ A2 B2]):
//   * k_tc_split writes, once per matrix, K-major FP32 planes: Re hi, Re lo, Im hi, Im lo
//     of the A operands (transposed: K contiguous per row of A) and the same plus -Im hi,
//     -Im lo of the B operands (as stored: K contiguous per column of B), K padded with
//     zeros to Kp = 32 k;
//   * one producer thread streams the planes of each 32-wide K slice into a two-stage
//     shared-memory ring with cp.async.bulk.tensor (128-byte swizzle, the layout the MMA
//     descriptors describe), each stage guarded by a "full" and an "empty" mbarrier.  The
//     B planes of a stage lie as [-Bi | Br | Bi] (hi, then lo), so the 128-row windows
//     W1 = [Br | Bi] and W2 = [-Bi | Br] are B operands of single MMAs:
//         [Re | Im](C) += Ar W1 + Ai W2;
//   * one thread issues tcgen05.mma (M = 128, N = 128, K = 8 per instruction, 6 per K
//     step: 3xTF32 of the two products) into one tensor-memory accumulator (Re: columns
//     0-63, Im: 64-127) and frees each stage with tcgen05.commit;
//   * the four warps read their 32 lanes (rows) back with tcgen05.ld and write C.
// Every wait is bounded (error flag, then the kernel carries on to release its tensor
// memory); tensor memory is allocated and freed by warp 0.
#include "kore_internal.cuh"
#include "kore_tma.cuh"
#include <algorithm>
#include <cstdio>
#include <vector>

namespace {

constexpr int kTcM = 128, kTcN = 64, kTcK = 32, kTcStages = 2, kTcThreads = 128;
constexpr int kPlanesA = 4, kPlanesB = 6;         // A: Re hi, Re lo, Im hi, Im lo; B: + -Im hi, -Im lo
constexpr int kPlaneA = kTcM * kTcK * 4;          // 16 KB: one plane of an A slice
constexpr int kPlaneB = kTcN * kTcK * 4;          // 8 KB
constexpr int kStageA = kPlanesA * kPlaneA;
constexpr int kStageBytes = kStageA + kPlanesB * kPlaneB;   // 112 KB
constexpr uint32_t kTmemCols = 2 * kTcN;          // [Re | Im] accumulator: columns [0, 64) and [64, 128)
constexpr size_t kTcSmem = (size_t)kTcStages * kStageBytes + 1024 + 128;
// Order of the B planes in a stage: [-Im hi][Re hi][Im hi][-Im lo][Re lo][Im lo]; stage
// slot of global plane p (Re hi, Re lo, Im hi, Im lo, -Im hi, -Im lo).
__host__ __device__ constexpr int slot_b(int p) {
    return p == 0 ? 1 : p == 1 ? 4 : p == 2 ? 2 : p == 3 ? 5 : p == 4 ? 0 : 3;
}

struct TcJob {
    int a1, b1, a2, b2;   // matrix indices into the A and B plane sets (a2 < 0: one product)
    float2 *C;            // column-major S x S
    float alpha;          // C = beta C + alpha (A1 B1 + A2 B2)
    int beta;
};

struct TcParams {
    CUtensorMap amap, bmap;   // planes {Kp, S, 4 * matrices}, boxes {32, 128, 1} and {32, 64, 1}
    const TcJob *jobs;
    int S, Kp, tiles_n;
    int *err;
};

// ----------------------------------------------------------------------------- tcgen05 PTX
__device__ __forceinline__ void tc_alloc(uint32_t *holder, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] B[smem]; accumulate = 0 overwrites D
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on `bar` once every MMA this thread issued before has completed
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive 32-bit columns of this warp's 32 lanes
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand in the 128-byte swizzled layout:
// rows of 128 bytes (32 TF32 of K), 8-row groups 1024 bytes apart.
//   [0,14) start address >> 4, [16,30) leading byte offset >> 4 (unused here: 1),
//   [32,46) stride byte offset >> 4 = 1024 >> 4, [46,48) version 1,
//   [49,52) base offset 0 (1024-byte aligned tiles), [61,64) layout 2 = 128-byte swizzle.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::tf32: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9,
// 10-12 = 2), no negation (bits 13, 14), both operands K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22 (N = 128: the [Re | Im] window), M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tf32_idesc() {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)((2 * kTcN) >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// ----------------------------------------------------------------------------- split planes
// planes[((m * P + p) * S + row) * Kp + k], p = Re hi, Re lo, Im hi, Im lo (P = 4, A
// operands) and -Im hi, -Im lo (P = 6, B operands).  TRANS (A operand): row = row of X,
// k = column of X.  !TRANS (B operand): row = column of X, k = row of X.  X is
// column-major S x S; k in [S, Kp) is zero.
template <bool TRANS>
__global__ void __launch_bounds__(256) k_tc_split(const float2 *const *__restrict__ src, int S, int Kp,
                                                  float *__restrict__ planes) {
    __shared__ float2 t[32][33];
    const int m = blockIdx.z;
    const float2 *X = src[m];
    const int k0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
    const int64_t plane = (int64_t)S * Kp;
    float *base = planes + (int64_t)m * (TRANS ? kPlanesA : kPlanesB) * plane;
    auto put = [&](int row, int k, float2 v) {
        const float rh = tf32_rna(v.x), ih = tf32_rna(v.y);
        const int64_t o = (int64_t)row * Kp + k;
        base[o] = rh;
        base[plane + o] = v.x - rh;
        base[2 * plane + o] = ih;
        base[3 * plane + o] = v.y - ih;
        if (!TRANS) {
            base[4 * plane + o] = -ih;
            base[5 * plane + o] = -(v.y - ih);
        }
    };
    if (TRANS) {
        // read X(r0 + tx, k0 + j) along its rows, write row r0 + j along k
        for (int j = ty; j < 32; j += 8) {
            const int r = r0 + tx, k = k0 + j;
            t[j][tx] = (r < S && k < S) ? X[r + (int64_t)k * S] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int j = ty; j < 32; j += 8) {
            const int r = r0 + j, k = k0 + tx;
            if (r < S && k < Kp) put(r, k, t[tx][j]);
        }
    } else {
        for (int j = ty; j < 32; j += 8) {
            const int n = r0 + j, k = k0 + tx;
            if (n < S && k < Kp) put(n, k, (k < S) ? X[k + (int64_t)n * S] : make_float2(0.f, 0.f));
        }
    }
}

// ----------------------------------------------------------------------------- GEMM
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_gemm(const __grid_constant__ TcParams P) {
    extern __shared__ unsigned char smem_raw[];
    // 1024-byte aligned stages (the 128-byte swizzle pattern repeats every 1024 bytes)
    unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kTcStages * kStageBytes);
    uint64_t *empty = full + kTcStages;
    uint64_t *accum = empty + kTcStages;
    uint32_t *holder = reinterpret_cast<uint32_t *>(accum + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TcJob job = P.jobs[blockIdx.y];
    const int tm = blockIdx.x / P.tiles_n, tn = blockIdx.x - tm * P.tiles_n;
    const int nk = P.Kp / kTcK;
    const int nstage = (job.a2 >= 0 ? 2 : 1) * nk;
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        mbar_fence_init();
    }
    if (warp == 0) tc_alloc(holder, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *holder;

    if (warp == 0) {
        if (lane == 0) {
            // producer: the four planes of A and of B for each 32-wide K slice
            for (int ks = 0; ks < nstage; ++ks) {
                const int s = ks % kTcStages;
                const uint32_t ph = (uint32_t)(ks / kTcStages) & 1u;
                if (!mbar_wait(&empty[s], ph ^ 1u)) atomicCAS(P.err, 0, KORE_DEVERR_FLAG);
                mbar_arrive_expect_tx(&full[s], kStageBytes);
                const int pair = ks / nk, kq = ks - pair * nk;
                const int ia = pair ? job.a2 : job.a1, ib = pair ? job.b2 : job.b1;
                unsigned char *sa = smem + (size_t)s * kStageBytes, *sb = sa + kStageA;
#pragma unroll
                for (int p = 0; p < kPlanesA; ++p)
                    tma_load_3d(sa + p * kPlaneA, &P.amap, &full[s], kq * kTcK, tm * kTcM, ia * kPlanesA + p);
#pragma unroll
                for (int p = 0; p < kPlanesB; ++p)
                    tma_load_3d(sb + slot_b(p) * kPlaneB, &P.bmap, &full[s], kq * kTcK, tn * kTcN, ib * kPlanesB + p);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            const uint32_t id = tf32_idesc();
            for (int ks = 0; ks < nstage; ++ks) {
                const int s = ks % kTcStages;
                const uint32_t ph = (uint32_t)(ks / kTcStages) & 1u;
                if (!mbar_wait(&full[s], ph)) atomicCAS(P.err, 0, KORE_DEVERR_FLAG);
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + (size_t)s * kStageBytes), sb = sa + kStageA;
#pragma unroll
                for (int k8 = 0; k8 < kTcK / 8; ++k8) {
                    uint64_t a[kPlanesA];
#pragma unroll
                    for (int p = 0; p < kPlanesA; ++p) a[p] = sw128_desc(sa + p * kPlaneA) + (uint64_t)(2 * k8);
                    // 128-row windows of the B planes (+ 32 bytes of K per step of 8)
                    const uint64_t w1h = sw128_desc(sb + 1 * kPlaneB) + (uint64_t)(2 * k8);   // [Br hi | Bi hi]
                    const uint64_t w2h = sw128_desc(sb + 0 * kPlaneB) + (uint64_t)(2 * k8);   // [-Bi hi | Br hi]
                    const uint64_t w1l = sw128_desc(sb + 4 * kPlaneB) + (uint64_t)(2 * k8);   // [Br lo | Bi lo]
                    const uint64_t w2l = sw128_desc(sb + 3 * kPlaneB) + (uint64_t)(2 * k8);   // [-Bi lo | Br lo]
                    const uint32_t acc = (ks == 0 && k8 == 0) ? 0u : 1u;
                    // [Re | Im] += Ar [Br | Bi]
                    tc_mma(tmem, a[0], w1h, id, acc);
                    tc_mma(tmem, a[0], w1l, id, 1u);
                    tc_mma(tmem, a[1], w1h, id, 1u);
                    // [Re | Im] += Ai [-Bi | Br]
                    tc_mma(tmem, a[2], w2h, id, 1u);
                    tc_mma(tmem, a[2], w2l, id, 1u);
                    tc_mma(tmem, a[3], w2h, id, 1u);
                }
                tc_commit(&empty[s]);   // the slot is free once these MMAs have read it
            }
            tc_commit(accum);
        }
        __syncwarp();
    }

    // epilogue: warp w holds rows 32 w .. 32 w + 31 of the tile in its tensor-memory lanes
    if (!mbar_wait(accum, 0)) atomicCAS(P.err, 0, KORE_DEVERR_FLAG);
    tc_fence_after();
    const int row = tm * kTcM + warp * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < kTcN; c0 += 16) {
        float re[16], im[16];
        tc_ld16(tl + (uint32_t)c0, re);
        tc_ld16(tl + (uint32_t)(kTcN + c0), im);
        tc_ld_wait();
        if (row < P.S) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = tn * kTcN + c0 + j;
                if (col < P.S) {
                    float2 *c = job.C + row + (int64_t)col * P.S;
                    float2 v = make_float2(job.alpha * re[j], job.alpha * im[j]);
                    if (job.beta) {
                        const float2 o = *c;
                        v.x += o.x;
                        v.y += o.y;
                    }
                    *c = v;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, kTmemCols);
}

// ----------------------------------------------------------------------------- host
int tc_kp(int S) { return (S + kTcK - 1) / kTcK * kTcK; }

// Splits srcA / srcB (device arrays of nA / nB matrix pointers, already on the device),
// encodes the tensor maps and runs the jobs (device array of njobs).
int tc_run(cudaStream_t st, int device, int S, const float2 *const *srcA, int nA, const float2 *const *srcB, int nB,
           const TcJob *jobs, int njobs, float *planes, int *err) {
    if (njobs == 0) return KORE_OK;
    if (nA > 65535 || nB > 65535) return KORE_EINVAL;
    const int Kp = tc_kp(S);
    float *pa = planes, *pb = planes + (int64_t)nA * kPlanesA * S * Kp;
    const dim3 sg(Kp / 32, kore_div_up(S, 32));
    k_tc_split<true><<<dim3(sg.x, sg.y, nA), dim3(32, 8), 0, st>>>(srcA, S, Kp, pa);
    k_tc_split<false><<<dim3(sg.x, sg.y, nB), dim3(32, 8), 0, st>>>(srcB, S, Kp, pb);
    KORE_LAUNCHED(2);
    TcParams P;
    const uint64_t da[3] = {(uint64_t)Kp, (uint64_t)S, (uint64_t)kPlanesA * nA};
    const uint64_t db[3] = {(uint64_t)Kp, (uint64_t)S, (uint64_t)kPlanesB * nB};
    const uint64_t sd[2] = {(uint64_t)Kp * 4, (uint64_t)S * Kp * 4};
    const uint32_t ba[3] = {kTcK, kTcM, 1}, bb[3] = {kTcK, kTcN, 1};
    KORE_TRY(kore_encode_f32_3d(&P.amap, pa, da, sd, ba, 1));
    KORE_TRY(kore_encode_f32_3d(&P.bmap, pb, db, sd, bb, 1));
    P.S = S;
    P.Kp = Kp;
    P.tiles_n = kore_div_up(S, kTcN);
    P.err = err;
    const int tiles = kore_div_up(S, kTcM) * P.tiles_n;
    KORE_TRY(kore_allow_max_dyn_smem(k_tc_gemm, device));
    for (int j0 = 0; j0 < njobs; j0 += 65535) {
        P.jobs = jobs + j0;
        k_tc_gemm<<<dim3(tiles, std::min(65535, njobs - j0)), kTcThreads, kTcSmem, st>>>(P);
        KORE_LAUNCHED(1);
    }
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

// FP64 reference of the self-test: C_ref(r, c) = beta C0 + alpha sum of the products
// and the magnitude bound sum |a| |b| (one thread per element).
__global__ void k_tc_ref(int S, const float2 *A, const float2 *B, const TcJob *jobs, int njobs, const float2 *C0,
                         double *err) {
    const int j = blockIdx.y;
    if (j >= njobs) return;
    const TcJob jb = jobs[j];
    const int64_t SS = (int64_t)S * S;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < SS; e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % S), c = (int)(e / S);
        double sr = 0, si = 0, mag = 0;
        for (int pr = 0; pr < 2; ++pr) {
            const int ia = pr ? jb.a2 : jb.a1, ib = pr ? jb.b2 : jb.b1;
            if (ia < 0) continue;
            for (int k = 0; k < S; ++k) {
                const float2 a = A[ia * SS + r + (int64_t)k * S], b = B[ib * SS + k + (int64_t)c * S];
                sr += (double)a.x * b.x - (double)a.y * b.y;
                si += (double)a.x * b.y + (double)a.y * b.x;
                mag += (fabs((double)a.x) + fabs((double)a.y)) * (fabs((double)b.x) + fabs((double)b.y));
            }
        }
        double rr = jb.alpha * sr, ri = jb.alpha * si;
        if (jb.beta) { rr += C0[j * SS + e].x; ri += C0[j * SS + e].y; }
        const float2 got = jb.C[e];
        const double d = fmax(fabs(got.x - rr), fabs(got.y - ri)) / fmax(mag, 1e-30);
        // max of non-negative doubles through their bit patterns
        atomicMax(reinterpret_cast<unsigned long long *>(err), (unsigned long long)__double_as_longlong(d));
    }
}

__global__ void k_tc_fill(float2 *x, int64_t n, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t h = (uint64_t)i * 0x9E3779B97F4A7C15ULL + seed;
        h ^= h >> 31; h *= 0xBF58476D1CE4E5B9ULL; h ^= h >> 27; h *= 0x94D049BB133111EBULL; h ^= h >> 31;
        const float u = (float)(h & 0xFFFFFF) / 16777216.f - 0.5f;
        const float v = (float)((h >> 24) & 0xFFFFFF) / 16777216.f - 0.5f;
        x[i] = make_float2(u, v);
    }
}

}  // namespace

// ----------------------------------------------------------------------------- factorisation use
int tc_upload_run(kore_plan *p, const std::vector<const float2 *> &src, int64_t nA, const std::vector<TcJob> &jobs);
// Bytes of the split planes and the job table for one reduction level's even-block update
// (levels >= 1) of `cap` shifts; the plan allocates the largest over its levels.
void kore_tc_level_bytes(const kore_plan *p, int cap, int64_t *plane_bytes, int64_t *table_bytes) {
    int64_t pl = 0, tb = 0;
    const int64_t S = p->S, Kp = tc_kp(p->S);
    for (int l = 0; l < p->nlev; ++l) {
        const int64_t ne = p->lev[l].neven, no = p->lev[l].nodd;
        // even update (levels >= 1): 2 neven A + 2 nodd B matrices, 3 neven jobs;
        // G, H and their refinement (every level): nodd A + 2 nodd B matrices, 2 nodd jobs
        // planes: 4 per A and 6 per B matrix
        const int64_t np_ = std::max(l > 0 ? 2 * ne * kPlanesA + 2 * no * kPlanesB : 0,
                                     no * kPlanesA + 2 * no * kPlanesB) * cap;
        const int64_t nm = std::max(l > 0 ? 2 * (ne + no) : 0, 3 * no) * cap;
        const int64_t nj = std::max(l > 0 ? 3 * ne : 0, 2 * no) * cap;
        pl = std::max(pl, np_ * S * Kp * 4);
        tb = std::max(tb, nm * 8 + nj * (int64_t)sizeof(TcJob) + 64);
    }
    *plane_bytes = pl;
    *table_bytes = tb;
}

// Even-block update of level l >= 1 for every shift (complex64 factors), the
// tensor-core form of k_even_gemm: D_i -= L_q H_jl + U_q G_jr;  L' = -L_q G_jl;
// U' = -U_q H_jr.
int kore_even_update_tc(kore_plan *p, const BcrLevel &lv) {
    const int S = p->S, ns = p->fw_n;
    const int64_t lo = p->fw_lo;   // shift sh of the factor window is shift lo + sh of the plan
    const int64_t SS = (int64_t)S * S;
    std::vector<const float2 *> src;   // A operands, then B operands
    std::vector<TcJob> jobs;
    const int64_t nA = 2 * (int64_t)lv.neven * ns, nB = 2 * (int64_t)lv.nodd * ns;
    src.reserve(nA + nB);
    for (int sh = 0; sh < ns; ++sh) {
        const float2 *LU = static_cast<const float2 *>(p->d_LU) + (lo + sh) * p->lu_stride();
        for (int e = 0; e < lv.neven; ++e) {
            src.push_back(LU + (lv.lu_L + 2 * e) * SS);   // A index (sh neven + e) 2 + 0: L_q
            src.push_back(LU + (lv.lu_U + 2 * e) * SS);   //                            + 1: U_q
        }
    }
    for (int sh = 0; sh < ns; ++sh) {
        const float2 *G = static_cast<const float2 *>(p->d_Gm) + (lo + sh) * p->f_stride();
        const float2 *H = static_cast<const float2 *>(p->d_Hm) + (lo + sh) * p->f_stride();
        for (int o = 0; o < lv.nodd; ++o) {
            const int64_t j = (int64_t)(2 * o + 1) * lv.stride;
            src.push_back(G + j * SS);                    // B index (sh nodd + o) 2 + 0: G_j
            src.push_back(H + j * SS);                    //                         + 1: H_j
        }
    }
    for (int sh = 0; sh < ns; ++sh) {
        float2 *LU = static_cast<float2 *>(p->d_LU) + (lo + sh) * p->lu_stride();
        float2 *Dw = static_cast<float2 *>(p->d_Dw) + (lo + sh) * p->f_stride();
        for (int e = 0; e < lv.neven; ++e) {
            const int q = 2 * e;
            const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
            const int aL = (sh * lv.neven + e) * 2, aU = aL + 1;
            const int bl = (sh * lv.nodd + e - 1) * 2, br = (sh * lv.nodd + e) * 2;   // + 0: G, + 1: H
            if (hasl || hasr) {
                TcJob j{-1, -1, -1, -1, Dw + (int64_t)q * lv.stride * SS, -1.f, 1};
                if (hasl) { j.a1 = aL; j.b1 = bl + 1; }
                if (hasr) {
                    if (j.a1 < 0) { j.a1 = aU; j.b1 = br; }
                    else { j.a2 = aU; j.b2 = br; }
                }
                jobs.push_back(j);
            }
            if (lv.lu_nL >= 0 && q >= 2) jobs.push_back(TcJob{aL, bl, -1, -1, LU + (lv.lu_nL + e) * SS, -1.f, 0});
            if (lv.lu_nU >= 0 && q + 2 < lv.Kl)
                jobs.push_back(TcJob{aU, br + 1, -1, -1, LU + (lv.lu_nU + e) * SS, -1.f, 0});
        }
    }
    (void)nB;
    return tc_upload_run(p, src, nA, jobs);
}

// R(k, c) += rs_k a_e for the level-0 couplings of the odd blocks (side 0: L_j into
// R_G, side 1: U_j into R_H), R_G and R_H at Rbase + shift * t_stride + o * 2 S^2 (+ S^2).
// CTA = (odd index o, side, shift); threads over the columns.
__global__ void k_add_couplings(const int *__restrict__ cc_ptr, const int *__restrict__ cc_row,
                                const int *__restrict__ cc_src, const double2 *__restrict__ aval,
                                const double *__restrict__ rscale, int S, int64_t np, float2 *Rbase,
                                int64_t t_stride) {
    const int64_t o = blockIdx.x, side = blockIdx.y, sh = blockIdx.z;
    const int64_t SS = (int64_t)S * S, j = 2 * o + 1;
    const int *ptr = cc_ptr + (2 * o + side) * (int64_t)(S + 1);
    const double *rs = rscale + sh * np + j * S;
    float2 *R = Rbase + sh * t_stride + o * 2 * SS + side * SS;
    for (int c = threadIdx.x; c < S; c += blockDim.x)
        for (int t = ptr[c]; t < ptr[c + 1]; ++t) {
            const int k = cc_row[t];
            const double2 a = rs[k] * aval[cc_src[t]];
            float2 &r = R[k + (int64_t)c * S];
            r = make_float2((float)((double)r.x + a.x), (float)((double)r.y + a.y));
        }
}

int tc_upload_run(kore_plan *p, const std::vector<const float2 *> &src, int64_t nA, const std::vector<TcJob> &jobs) {
    const size_t pbytes = src.size() * sizeof(void *), jbytes = jobs.size() * sizeof(TcJob);
    unsigned char *tab = static_cast<unsigned char *>(p->d_tctab);
    KORE_CUDA_TRY(cudaMemcpyAsync(tab, src.data(), pbytes, cudaMemcpyHostToDevice, p->stream));
    KORE_CUDA_TRY(cudaMemcpyAsync(tab + pbytes, jobs.data(), jbytes, cudaMemcpyHostToDevice, p->stream));
    const float2 *const *dsrc = reinterpret_cast<const float2 *const *>(tab);
    return tc_run(p->stream, p->device, p->S, dsrc, (int)nA, dsrc + nA, (int)(src.size() - nA),
                  reinterpret_cast<const TcJob *>(tab + pbytes), (int)jobs.size(), static_cast<float *>(p->d_tcplanes),
                  p->d_err);
}

// G_j = D_j^-1 L_j and H_j = D_j^-1 U_j of the odd blocks of a level for every shift
// (complex64 factors), on the tensor cores, with one step of refinement:
//     G0 = D^-1 L,   R = L - D G0,   G = G0 + D^-1 R
// (D is the row-scaled diagonal block, D^-1 its Gauss-Jordan inverse).  The product with
// an explicit inverse loses accuracy where D^-1 L cancels; the refinement step gives
// the columns of G the accuracy of a stable solve, which keeps the FP64 refinement of
// the solves at two to three corrections.  Level >= 1: dense L, U in the coupling
// store (the odd blocks' L, U are not read again, so R overwrites them).  Level 0:
// G0 and H0 come from the sparse couplings (k_gh_l0); R goes to the Gauss-Jordan work
// area T, free after the extraction.
int kore_gh_update_tc(kore_plan *p, const BcrLevel &lv, int level0) {
    const int S = p->S, ns = p->fw_n;
    const int64_t lo = p->fw_lo;   // shift sh of the factor window is shift lo + sh of the plan
    const int64_t SS = (int64_t)S * S, no = lv.nodd;
    float2 *Dinv = static_cast<float2 *>(p->d_Dinv), *Dw = static_cast<float2 *>(p->d_Dw);
    float2 *G = static_cast<float2 *>(p->d_Gm), *H = static_cast<float2 *>(p->d_Hm);
    float2 *LU = static_cast<float2 *>(p->d_LU), *T = static_cast<float2 *>(p->d_T);
    auto blk = [&](float2 *base, int sh, int64_t o) {
        return base + (lo + sh) * p->f_stride() + (2 * o + 1) * lv.stride * SS;
    };
    // residual storage of (shift, odd o, side)
    auto rstore = [&](int sh, int64_t o, int side) -> float2 * {
        if (level0) return T + (lo + sh) * p->t_stride() + o * 2 * SS + side * SS;
        return LU + (lo + sh) * p->lu_stride() + ((side ? lv.lu_U : lv.lu_L) + 2 * o + 1) * SS;
    };
    auto hasr = [&](int64_t o) { return 2 * o + 2 < lv.Kl; };
    std::vector<const float2 *> src;
    std::vector<TcJob> jobs;
    // stage 1 (levels >= 1): G0 = D^-1 L, H0 = D^-1 U
    if (!level0) {
        for (int sh = 0; sh < ns; ++sh)
            for (int64_t o = 0; o < no; ++o) src.push_back(blk(Dinv, sh, o));
        for (int sh = 0; sh < ns; ++sh)
            for (int64_t o = 0; o < no; ++o) { src.push_back(rstore(sh, o, 0)); src.push_back(rstore(sh, o, 1)); }
        for (int sh = 0; sh < ns; ++sh)
            for (int64_t o = 0; o < no; ++o) {
                const int a = (int)(sh * no + o);
                jobs.push_back(TcJob{a, 2 * a, -1, -1, blk(G, sh, o), 1.f, 0});
                if (hasr(o)) jobs.push_back(TcJob{a, 2 * a + 1, -1, -1, blk(H, sh, o), 1.f, 0});
            }
        KORE_TRY(tc_upload_run(p, src, ns * no, jobs));
    }
    // stage 2: R = L - D G0 (level 0: R = -D G0, then + L from the sparse couplings)
    src.clear();
    jobs.clear();
    for (int sh = 0; sh < ns; ++sh)
        for (int64_t o = 0; o < no; ++o) src.push_back(blk(Dw, sh, o));
    for (int sh = 0; sh < ns; ++sh)
        for (int64_t o = 0; o < no; ++o) { src.push_back(blk(G, sh, o)); src.push_back(blk(H, sh, o)); }
    for (int sh = 0; sh < ns; ++sh)
        for (int64_t o = 0; o < no; ++o) {
            const int a = (int)(sh * no + o);
            const int beta = level0 ? 0 : 1;
            jobs.push_back(TcJob{a, 2 * a, -1, -1, rstore(sh, o, 0), -1.f, beta});
            if (hasr(o)) jobs.push_back(TcJob{a, 2 * a + 1, -1, -1, rstore(sh, o, 1), -1.f, beta});
        }
    KORE_TRY(tc_upload_run(p, src, ns * no, jobs));
    if (level0) {
        k_add_couplings<<<dim3((unsigned)no, 2, ns), 256, 0, p->stream>>>(p->d_cc_ptr, p->d_cc_row, p->d_cc_src,
                                                                          p->d_aval, p->d_rscale + lo * p->np, S,
                                                                          p->np, T + lo * p->t_stride(),
                                                                          p->t_stride());
        KORE_LAUNCHED(1);
    }
    // stage 3: G = G0 + D^-1 R
    src.clear();
    jobs.clear();
    for (int sh = 0; sh < ns; ++sh)
        for (int64_t o = 0; o < no; ++o) src.push_back(blk(Dinv, sh, o));
    for (int sh = 0; sh < ns; ++sh)
        for (int64_t o = 0; o < no; ++o) { src.push_back(rstore(sh, o, 0)); src.push_back(rstore(sh, o, 1)); }
    for (int sh = 0; sh < ns; ++sh)
        for (int64_t o = 0; o < no; ++o) {
            const int a = (int)(sh * no + o);
            jobs.push_back(TcJob{a, 2 * a, -1, -1, blk(G, sh, o), 1.f, 1});
            if (hasr(o)) jobs.push_back(TcJob{a, 2 * a + 1, -1, -1, blk(H, sh, o), 1.f, 1});
        }
    return tc_upload_run(p, src, ns * no, jobs);
}

extern "C" int kore_tc_selftest(int device, int S, int nmat, double *max_rel_err) {
    if (!max_rel_err || S <= 0 || S > 1024 || nmat < 2 || nmat > 64) return KORE_EINVAL;
    int prev = -1;
    cudaGetDevice(&prev);
    KORE_CUDA_TRY(cudaSetDevice(device));
    const int64_t SS = (int64_t)S * S, Kp = tc_kp(S);
    float2 *A = nullptr, *B = nullptr, *C = nullptr, *C0 = nullptr;
    float *planes = nullptr;
    unsigned char *tab = nullptr;
    double *err = nullptr;
    int *flag = nullptr;
    int rc = KORE_OK;
    auto ck = [&](cudaError_t e) { if (e != cudaSuccess && rc == KORE_OK) rc = (e == cudaErrorMemoryAllocation) ? KORE_ENOMEM : KORE_ECUDA; };
    ck(cudaMalloc(&A, nmat * SS * sizeof(float2)));
    ck(cudaMalloc(&B, nmat * SS * sizeof(float2)));
    ck(cudaMalloc(&C, nmat * SS * sizeof(float2)));
    ck(cudaMalloc(&C0, nmat * SS * sizeof(float2)));
    ck(cudaMalloc(&planes, (size_t)nmat * (kPlanesA + kPlanesB) * S * Kp * sizeof(float)));
    ck(cudaMalloc(&tab, (size_t)2 * nmat * 8 + (size_t)nmat * sizeof(TcJob)));
    ck(cudaMalloc(&err, sizeof(double)));
    ck(cudaMalloc(&flag, sizeof(int)));
    if (rc == KORE_OK) {
        k_tc_fill<<<256, 256>>>(A, nmat * SS, 1);
        k_tc_fill<<<256, 256>>>(B, nmat * SS, 2);
        k_tc_fill<<<256, 256>>>(C, nmat * SS, 3);
        ck(cudaMemcpy(C0, C, nmat * SS * sizeof(float2), cudaMemcpyDeviceToDevice));
        ck(cudaMemset(err, 0, sizeof(double)));
        ck(cudaMemset(flag, 0, sizeof(int)));
        std::vector<const float2 *> src;
        for (int m = 0; m < nmat; ++m) src.push_back(A + m * SS);
        for (int m = 0; m < nmat; ++m) src.push_back(B + m * SS);
        // job m: even m: C_m = A_m B_m;  odd m: C_m -= A_m B_m + A_{m-1} B_{m+1 mod n}
        std::vector<TcJob> jobs;
        for (int m = 0; m < nmat; ++m) {
            if (m % 2 == 0) jobs.push_back(TcJob{m, m, -1, -1, C + m * SS, 1.f, 0});
            else jobs.push_back(TcJob{m, m, m - 1, (m + 1) % nmat, C + m * SS, -1.f, 1});
        }
        ck(cudaMemcpy(tab, src.data(), src.size() * 8, cudaMemcpyHostToDevice));
        ck(cudaMemcpy(tab + src.size() * 8, jobs.data(), jobs.size() * sizeof(TcJob), cudaMemcpyHostToDevice));
        const float2 *const *dsrc = reinterpret_cast<const float2 *const *>(tab);
        const TcJob *djobs = reinterpret_cast<const TcJob *>(tab + src.size() * 8);
        if (rc == KORE_OK) rc = tc_run(0, device, S, dsrc, nmat, dsrc + nmat, nmat, djobs, nmat, planes, flag);
        if (rc == KORE_OK) {
            k_tc_ref<<<dim3(64, nmat), 256>>>(S, A, B, djobs, nmat, C0, err);
            ck(cudaGetLastError());
            ck(cudaDeviceSynchronize());
            int h = 0;
            ck(cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost));
            ck(cudaMemcpy(max_rel_err, err, sizeof(double), cudaMemcpyDeviceToHost));
            if (rc == KORE_OK && h != 0) rc = KORE_ETIMEOUT;
        }
    }
    cudaFree(A); cudaFree(B); cudaFree(C); cudaFree(C0); cudaFree(planes); cudaFree(tab); cudaFree(err); cudaFree(flag);
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}
