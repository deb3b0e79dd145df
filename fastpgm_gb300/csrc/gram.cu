// Level-0 pair counts on the tensor cores.
//
// Level 0 of PC-stable tests every pair x < y of one dataset without a conditioning set
// (PCStable.cpp:133-177); each test needs the pair's joint table N[i][j] = #{t : x_t = i,
// y_t = j} (Counts2D::FillTable, CellTable.cpp:430-455).  All of those tables at once are
// one contraction: with H the one-hot matrix of the samples -- row (v, s) holds 1 where
// variable v takes state s -- the Gram matrix G = H H^T holds N_xy in the block of rows of x
// and columns of y, and the one-way counts N_x[i] on the diagonal.
//
//   onehot_kernel  H[r][t] = 1.0 (E4M3 0x38) or 0, rows packed variable after variable,
//                  samples along K padded with zeros to a multiple of 128
//   gram_kernel    the upper-triangle 128x128 tiles of G: TMA (cp.async.bulk.tensor, 128-byte
//                  swizzle) stages 128x128-byte tiles of H into shared memory, one thread
//                  issues tcgen05.mma.kind::f8f6f4 (E4M3 x E4M3, FP32 accumulation in TMEM),
//                  the four warps read the accumulator back with tcgen05.ld and store int32.
//                  Products of one-hot entries are 0 or 1, so every partial sum is an integer
//                  below 2^24 (at most the sample count): exact in FP32.  When there are few
//                  tiles, K is split over CTAs and the partial counts are added with
//                  reductions into a zeroed G.
//
// Every mbarrier wait is bounded; on a timeout the kernel raises *err, stops issuing, waits
// (bounded) for the copies it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "fastpgm_gb300.h"
#include "engine_internal.h"

namespace fpgm {
namespace {

constexpr int kTile = 128;                 // rows of a G tile (M = N = 128), bytes of a K block
constexpr int kStages = 6;                 // TMA ring: 6 x (16 KB A + 16 KB B)
constexpr int kStageBytes = 2 * kTile * kTile;
constexpr int kGramSmem = kStages * kStageBytes + 1024;  // + 1024-byte alignment slack
constexpr int kGramThreads = 128;
constexpr long long kSpinLimit = 1ll << 26;  // mbarrier polls before a wait counts as hung
constexpr uint8_t kOne = 0x38;              // 1.0 in E4M3

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the completion of the phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (long long i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 bytes
// apart (SBO), version 1 (bits 46-47), layout SWIZZLE_128B (2 in bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                     // LBO (unused for swizzled K-major)
    d |= (uint64_t)((1024 >> 4) & 0x3FFF) << 32;  // SBO
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f8f6f4: D F32 (bits 4-5 = 1), A and B E4M3 (0), both
// K-major, N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(kTile >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);

__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// One-hot rows: thread per (variable, 16 samples); row_off[v] is v's first row.
__global__ void onehot_kernel(const uint8_t *cols, const int64_t *var_off, const uint8_t *card, const int32_t *row_off,
                              int n, int64_t S, int64_t K_pad, uint8_t *H) {
    const int64_t nvec = K_pad >> 4;
    const int64_t total = (int64_t)n * nvec;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int v = (int)(i / nvec);
        const int64_t t = i - (int64_t)v * nvec;
        uint32_t w[4] = {0, 0, 0, 0};
        if (16 * t < S) {
            const uint4 c = __ldg(reinterpret_cast<const uint4 *>(cols + var_off[v]) + t);
            w[0] = c.x;
            w[1] = c.y;
            w[2] = c.z;
            w[3] = c.w;
            // samples at or beyond S inside the last vector are not data
            const int64_t valid = S - 16 * t;
            if (valid < 16)
                for (int b = (int)valid; b < 16; ++b) w[b >> 2] |= 0xFFu << (8 * (b & 3));  // no state 255 row
        }
        const int c = card[v];
        uint8_t *dst = H + (int64_t)row_off[v] * K_pad + 16 * t;
        for (int s = 0; s < c; ++s) {
            uint32_t o[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t r = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) r |= (((w[q] >> (8 * b)) & 0xFFu) == (uint32_t)s ? (uint32_t)kOne : 0u) << (8 * b);
                o[q] = r;
            }
            if (16 * t >= S) o[0] = o[1] = o[2] = o[3] = 0;
            *reinterpret_cast<uint4 *>(dst + (int64_t)s * K_pad) = make_uint4(o[0], o[1], o[2], o[3]);
        }
    }
}

struct GramArgs {
    int32_t *G;       // [R_pad][R_pad]; upper tiles written (K split: added into zeros)
    int32_t R_pad;
    int32_t n_rt;     // row tiles
    int32_t kblocks;  // K_pad / 128
    int32_t ksplit;
    unsigned long long *err;
};

// Upper-triangle tile t -> (I, J), I <= J, row by row.
__device__ __forceinline__ void tile_of(int t, int n, int &I, int &J) {
    int i = 0;
    while (t >= n - i) {
        t -= n - i;
        ++i;
    }
    I = i;
    J = i + t;
}

__global__ void __launch_bounds__(kGramThreads, 1) gram_kernel(const __grid_constant__ CUtensorMap tmap, GramArgs g) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accf;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int t = blockIdx.x / g.ksplit, split = blockIdx.x - t * g.ksplit;
    int I, J;
    tile_of(t, g.n_rt, I, J);
    const int kb0 = (int)((int64_t)split * g.kblocks / g.ksplit);
    const int kb1 = (int)((int64_t)(split + 1) * g.kblocks / g.ksplit);
    const int nk = kb1 - kb0;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&accf, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(kTile)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    int issued = 0;  // producer: stages loaded
    if (warp == 0 && lane == 0) {
        for (int i = 0; i < nk; ++i) {
            const int st = i % kStages;
            if (i >= kStages && !mbar_wait(&empty[st], ((i / kStages) & 1) ^ 1)) {
                atomicExch(&s_abort, 1);
                break;
            }
            if (*(volatile int *)&s_abort) break;
            uint8_t *a = base + st * kStageBytes;
            mbar_expect_tx(&full[st], kStageBytes);
            tma_load_2d(a, &tmap, &full[st], (kb0 + i) * kTile, I * kTile);
            tma_load_2d(a + kTile * kTile, &tmap, &full[st], (kb0 + i) * kTile, J * kTile);
            ++issued;
        }
        // copies issued and never consumed (abort): wait for them before the CTA leaves
        if (*(volatile int *)&s_abort) {
            const int lo = issued > kStages ? issued - kStages : 0;
            for (int i = lo; i < issued; ++i) mbar_wait(&full[i % kStages], (i / kStages) & 1);
        }
    } else if (warp == 1 && lane == 0) {
        bool ok = true;
        for (int i = 0; i < nk; ++i) {
            const int st = i % kStages;
            if (!mbar_wait(&full[st], (i / kStages) & 1) || *(volatile int *)&s_abort) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smem_u32(base + st * kStageBytes);
            const uint64_t da = smem_desc(a), db = smem_desc(a + kTile * kTile);
#pragma unroll
            for (int kk = 0; kk < kTile / 32; ++kk)  // K = 32 bytes per instruction
                mma_f8(tmem, da + 2 * kk, db + 2 * kk, (i | kk) != 0);
            mma_commit(&empty[st]);
        }
        if (!ok) atomicExch(&s_abort, 1);
        mma_commit(&accf);  // arrives once every MMA issued above has completed
    }
    __syncwarp();
    // epilogue: warp w holds accumulator rows 32w .. 32w+31 (TMEM lanes)
    const bool acc_ok = mbar_wait(&accf, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!acc_ok) atomicExch(&s_abort, 1);
    __syncthreads();
    if (!s_abort && nk > 0) {
        const int row = I * kTile + warp * 32 + lane;
        int32_t *dst = g.G + (int64_t)row * g.R_pad + (int64_t)J * kTile;
        for (int c0 = 0; c0 < kTile; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            int v[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = __float2int_rn(__uint_as_float(r[j]));
            if (g.ksplit == 1) {
#pragma unroll
                for (int j = 0; j < 32; j += 4)
                    *reinterpret_cast<int4 *>(dst + c0 + j) = make_int4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (v[j]) atomicAdd(dst + c0 + j, v[j]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (s_abort && tid == 0) atomicExch(g.err, 1ull);
    if (warp == 2)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTile) : "memory");
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

#define GCK(call)                                                                                          \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return set_error(e_ == cudaErrorMemoryAllocation ? FPGM_ERR_OOM : FPGM_ERR_CUDA, "%s failed: %s", \
                             #call, cudaGetErrorString(e_));                                               \
    } while (0)

}  // namespace

struct GramLevel0 {
    int n = 0, R = 0, R_pad = 0, n_rt = 0, kblocks = 0, ksplit = 1, num_sms = 0, maxc = 1;
    int64_t S = 0, K_pad = 0;
    uint8_t *H = nullptr;
    size_t H_bytes = 0;
    int32_t *G = nullptr;
    size_t G_bytes = 0;
    int32_t *row_off = nullptr;
    size_t row_bytes = 0;
    const uint8_t *cols = nullptr;
    const int64_t *var_off = nullptr;
    const uint8_t *card = nullptr;
    CUtensorMap map;  // 64-byte aligned by its type
    bool attr_set = false;
};

GramLevel0 *gram_create() { return new GramLevel0(); }

void gram_destroy(GramLevel0 *g) {
    if (!g) return;
    dev_free(g->H, g->H_bytes);
    dev_free(g->G, g->G_bytes);
    dev_free(g->row_off, g->row_bytes);
    delete g;
}

static int grow(void **p, size_t *have, size_t need) {
    if (need <= *have) return FPGM_OK;
    dev_free(*p, *have);
    *p = nullptr;
    *have = 0;
    RET_IF(dev_alloc(p, need));
    *have = need;
    return FPGM_OK;
}

int gram_plan(GramLevel0 *g, int n, const uint8_t *h_card, int64_t S, const uint8_t *d_cols, const int64_t *d_var_off,
              const uint8_t *d_card, int num_sms, cudaStream_t stream, bool *ok) {
    *ok = false;
    int R = 0, maxc = 0;
    std::vector<int32_t> off(n + 1);
    for (int v = 0; v < n; ++v) {
        off[v] = R;
        R += h_card[v];
        maxc = std::max(maxc, (int)h_card[v]);
    }
    off[n] = R;
    // pair tables are scored by one warp in its 12 KB shared slice; the Gram matrix must fit
    if (maxc * maxc + 2 * maxc + 1 > 3000 || R > 32768 || S < 1 || S > (1 << 24) - 1) return FPGM_OK;
    g->n = n;
    g->maxc = maxc;
    g->R = R;
    g->R_pad = (R + kTile - 1) / kTile * kTile;
    g->n_rt = g->R_pad / kTile;
    g->S = S;
    g->K_pad = (S + kTile - 1) / kTile * kTile;
    g->kblocks = (int)(g->K_pad / kTile);
    g->num_sms = num_sms;
    const int tiles = g->n_rt * (g->n_rt + 1) / 2;
    // K split so that the grid holds about two CTAs per SM, each over at least 16 K blocks
    int ks = std::max(1, (2 * num_sms + tiles - 1) / tiles);
    ks = std::min(ks, std::max(1, g->kblocks / 16));
    g->ksplit = ks;
    g->cols = d_cols;
    g->var_off = d_var_off;
    g->card = d_card;
    RET_IF(grow(reinterpret_cast<void **>(&g->H), &g->H_bytes, (size_t)g->R_pad * g->K_pad));
    RET_IF(grow(reinterpret_cast<void **>(&g->G), &g->G_bytes, (size_t)g->R_pad * g->R_pad * 4));
    RET_IF(grow(reinterpret_cast<void **>(&g->row_off), &g->row_bytes, (size_t)(n + 1) * 4));
    GCK(cudaMemcpyAsync(g->row_off, off.data(), (size_t)(n + 1) * 4, cudaMemcpyHostToDevice, stream));
    // rows past R stay zero
    GCK(cudaMemsetAsync(g->H + (size_t)R * g->K_pad, 0, (size_t)(g->R_pad - R) * g->K_pad, stream));
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    GCK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (!fn || q != cudaDriverEntryPointSuccess)
        return set_error(FPGM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[2] = {(cuuint64_t)g->K_pad, (cuuint64_t)g->R_pad};
    const cuuint64_t strides[1] = {(cuuint64_t)g->K_pad};  // bytes between rows (multiple of 128)
    const cuuint32_t box[2] = {kTile, kTile};
    const cuuint32_t estr[2] = {1, 1};
    CUresult cr = reinterpret_cast<EncodeTiled>(fn)(&g->map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, g->H, dims, strides,
                                                     box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(FPGM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)cr);
    if (!g->attr_set) {
        GCK(cudaFuncSetAttribute(gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmem));
        g->attr_set = true;
    }
    *ok = true;
    return FPGM_OK;
}

int gram_run(GramLevel0 *g, cudaStream_t stream, unsigned long long *err, int *launches) {
    const int64_t total = (int64_t)g->n * (g->K_pad >> 4);
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)g->num_sms * 16);
    onehot_kernel<<<blocks, 256, 0, stream>>>(g->cols, g->var_off, g->card, g->row_off, g->n, g->S, g->K_pad, g->H);
    GCK(cudaGetLastError());
    if (g->ksplit > 1) GCK(cudaMemsetAsync(g->G, 0, (size_t)g->R_pad * g->R_pad * 4, stream));
    GramArgs a;
    a.G = g->G;
    a.R_pad = g->R_pad;
    a.n_rt = g->n_rt;
    a.kblocks = g->kblocks;
    a.ksplit = g->ksplit;
    a.err = err;
    const int tiles = g->n_rt * (g->n_rt + 1) / 2;
    gram_kernel<<<tiles * g->ksplit, kGramThreads, kGramSmem, stream>>>(g->map, a);
    GCK(cudaGetLastError());
    if (launches) *launches += 2;
    return FPGM_OK;
}

const int32_t *gram_counts(const GramLevel0 *g) { return g->G; }
const int32_t *gram_row_off(const GramLevel0 *g) { return g->row_off; }
int gram_ld(const GramLevel0 *g) { return g->R_pad; }
int gram_slice_ints(const GramLevel0 *g) { return (g->maxc * g->maxc + 2 * g->maxc + 1 + 15) & ~15; }
double gram_flops(const GramLevel0 *g) {
    const double tiles = (double)g->n_rt * (g->n_rt + 1) / 2;
    return tiles * 2.0 * kTile * kTile * (double)g->K_pad;
}

}  // namespace fpgm
