// mdg_learned_tc.cu -- tensor-core (tcgen05) inference kernel of the
// learned slow force's MLP.
//
// CTAs of 4 warps (two per SM) walk 128-atom tiles.  Per tile, three layers:
//   D1[128 x 128] = X[128 x 64]   W1      (4 MMAs of K = 16)
//   D2[128 x 128] = H1[128 x 128] W2      (8 MMAs)
//   D3[128 x 16]  = H2[128 x 128] W3      (8 MMAs)
// tcgen05.mma.cta_group::1.kind::f16 (BF16 operands from shared memory,
// FP32 accumulators in tensor memory), issued by one thread and committed
// to an mbarrier.  Each warp then reads its 32 accumulator lanes (one atom
// per thread) with tcgen05.ld, adds the bias, applies SiLU, and writes the
// BF16 activations back to shared memory as the next layer's A operand.
// The last epilogue forms G_i = sum_b C_ib S_ib.
//
// Operand layout (shared memory and the prepared global weight copy): no
// swizzle, K-major, 8 x 16-byte core matrices, K-chunk-major: element
// (r, k) of an operand with R rows sits at byte
//     ((k / 8) * (R / 8) + r / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so the descriptor's leading-dimension offset (next 8 columns of K) is
// R * 16 bytes and its stride-dimension offset (next 8 rows) is 128 bytes.
//
// The weight images and each tile's features (stored in this layout by the
// feature kernel) arrive by bulk copies (cp.async.bulk) on a second
// mbarrier; the next tile's features load while the current tile's
// epilogues run.  Every mbarrier wait is bounded by wall time (1 s on the
// GPU's global timer); a wait that gives up raises MDG_ERR_TIMEOUT, waits
// (bounded the same way) for the MMAs and copies it started and has not
// seen complete, frees the tensor memory and leaves.
#include <cuda_bf16.h>

#include "mdg_internal.cuh"

namespace mdg {
namespace {

constexpr int kTcThreads = 128;
constexpr int kTmemCols = 256;
constexpr int kOffW1 = 0;                              // W1^T: 128 x 64
constexpr int kOffW2 = kOffW1 + kLsHidden * kLsFeat * 2;  // W2^T: 128 x 128
constexpr int kOffW3 = kOffW2 + kLsHidden * kLsHidden * 2;  // W3^T: 16 x 128
constexpr int kOffX = kOffW3 + kLsVec * kLsHidden * 2;   // X: 128 x 64
constexpr int kOffH = kOffX + kLsTile * kLsFeat * 2;     // H1 / H2: 128 x 128
constexpr int kOffB = kOffH + kLsTile * kLsHidden * 2;   // b1, b2, b3
constexpr int kOffBar = kOffB + 4 * (2 * kLsHidden + kLsVec + 4);
constexpr int kTcSmem = kOffBar + 32;  // MMA barrier, copy barrier, tensor-memory address
constexpr int kXBytes = kLsTile * kLsFeat * 2;
constexpr int kWtcBytes = kOffX;  // the three weight images, as laid out in global memory
// (two CTAs per SM: 2 x 256 tensor-memory columns fill the SM's 512)
constexpr int kTcSmemAlloc = (kTcSmem + 1023) / 1024 * 1024;
static_assert(kTcSmem <= kTcSmemAlloc, "shared memory");
static_assert(kWtcBytes / 2 == kLsWb, "weight image size");

__host__ __device__ constexpr int tc_off(int r, int k, int R) { return ls_tc_off(r, k, R); }

__device__ __forceinline__ uint16_t to_bf16(float v) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
// z sigmoid(z), as the SIMT kernels compute it
__device__ __forceinline__ float silu_f(float z) {
    return __fdividef(z, 1.0f + __expf(-fmaxf(z, -80.0f)));
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, leading / stride byte offsets,
// descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// A and B BF16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17,
// M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

// bulk copy global -> shared, completing on the mbarrier's transaction count
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                          uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits until the mbarrier phase of `parity` completes, for at most limit_ns
// of wall time (the GPU's global nanosecond timer); false when it gave up.
// Each try_wait may suspend the thread for a while, so the limit is taken
// from the clock, not from a count of tries (a count of 2^30 tries stays as
// a backstop should the timer not advance).
constexpr uint64_t kWaitNs = 1000000000ull;     // 1 s: every wait of a normal launch
constexpr uint64_t kTestWaitNs = 10000000ull;   // 10 ms: the first wait under the wait test
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          uint64_t limit_ns = kWaitNs) {
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 30); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 15u) == 15u && global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// bias + SiLU of this thread's 128 accumulators (columns col0..col0+127),
// BF16 into row t of the H operand
__device__ __forceinline__ void epilogue_hidden(uint32_t taddr, const float *bias, uint16_t *H,
                                                int t) {
#pragma unroll 1
    for (int cb = 0; cb < kLsHidden / 32; ++cb) {
        float v[32];
        tmem_ld32(taddr + cb * 32, v);
#pragma unroll
        for (int c8 = 0; c8 < 4; ++c8) {
            unsigned h[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int c = cb * 32 + c8 * 8 + 2 * u;
                h[u] = (unsigned)to_bf16(silu_f(v[c8 * 8 + 2 * u] + bias[c])) |
                       ((unsigned)to_bf16(silu_f(v[c8 * 8 + 2 * u + 1] + bias[c + 1])) << 16);
            }
            *(uint4 *)(H + tc_off(t, cb * 32 + c8 * 8, kLsTile)) = make_uint4(h[0], h[1], h[2], h[3]);
        }
    }
}

__global__ void __launch_bounds__(kTcThreads, 2)
    k_ls_mlp_tc(Learned L, int n_rows, int slot, int *status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int t = threadIdx.x, w = t >> 5;
    uint16_t *Hs = (uint16_t *)(sm + kOffH);
    float *sb = (float *)(sm + kOffB);
    uint32_t *tslot = (uint32_t *)(sm + kOffBar + 16);
    const uint32_t bar = smem_u32(sm + kOffBar), tbar = smem_u32(sm + kOffBar + 8);
    const int n_tiles = n_rows / kLsTile;
    const uint16_t *X = L.xb[slot];
    for (int e = t; e < kLsHidden; e += kTcThreads) {
        sb[e] = L.params[kLsB1 + e];
        sb[kLsHidden + e] = L.params[kLsB2 + e];
    }
    if (t < kLsVec) sb[2 * kLsHidden + t] = L.params[kLsB3 + t];
    // wait test (mdg_learned_wait_test): the first transaction is withheld,
    // so the copy barrier's first phase never completes and the first wait
    // runs out after kTestWaitNs; no copy and no MMA is in flight then
    const bool wait_test = L.tc_wait_test != 0;
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the weight images and the first tile's features, one transaction
        const int tile0 = blockIdx.x;
        if (!wait_test) {
            expect_tx(tbar, kWtcBytes + (tile0 < n_tiles ? kXBytes : 0));
            bulk_load(smem_u32(sm), L.wb + kLsWb, kWtcBytes, tbar);
            if (tile0 < n_tiles)
                bulk_load(smem_u32(sm + kOffX), X + (size_t)tile0 * kLsTile * kLsFeat, kXBytes,
                          tbar);
        }
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = *tslot;
    const uint32_t lane_base = (uint32_t)(32 * w) << 16;
    const float scale = L.params[kLsScale];
    const uint32_t a_x = smem_u32(sm + kOffX), a_h = smem_u32(Hs);
    const uint32_t a_w1 = smem_u32(sm + kOffW1), a_w2 = smem_u32(sm + kOffW2),
                   a_w3 = smem_u32(sm + kOffW3);
    constexpr uint32_t kLbo128 = kLsTile * 16, kLbo16 = kLsVec * 16, kSbo = 128;
    constexpr uint32_t id128 = idesc_bf16(128, 128), id16 = idesc_bf16(128, 16);
    uint32_t phase = 0, tphase = 0;
    // copies and MMAs this CTA has started and not yet seen complete: what a
    // CTA that gives up must wait for before it frees the tensor memory
    bool ok = true, copy_pending = !wait_test, mma_pending = false;
    bool first_wait = true;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int row = tile * kLsTile + t;
        // this tile's features (and, the first time, the weights) landed
        ok = mbar_wait(tbar, tphase, (first_wait && wait_test) ? kTestWaitNs : kWaitNs);
        first_wait = false;
        ok = __syncthreads_and(ok);
        if (!ok) break;
        tphase ^= 1;
        copy_pending = false;
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kLsFeat / 16; ++ks)
                mma_bf16(tm, sdesc(a_x + ks * 2 * kLbo128, kLbo128, kSbo),
                         sdesc(a_w1 + ks * 2 * kLbo128, kLbo128, kSbo), id128, ks);
            mma_commit(bar);
        }
        mma_pending = true;
        ok = mbar_wait(bar, phase);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        mma_pending = false;
        phase ^= 1;
        fence_after();
        const int next = tile + gridDim.x;
        if (t == 0 && next < n_tiles) {  // the layer-1 MMAs are done with X
            expect_tx(tbar, kXBytes);
            bulk_load(a_x, X + (size_t)next * kLsTile * kLsFeat, kXBytes, tbar);
        }
        copy_pending = next < n_tiles;
        epilogue_hidden(tm + lane_base, sb, Hs, t);
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kLsHidden / 16; ++ks)
                mma_bf16(tm + kLsHidden, sdesc(a_h + ks * 2 * kLbo128, kLbo128, kSbo),
                         sdesc(a_w2 + ks * 2 * kLbo128, kLbo128, kSbo), id128, ks);
            mma_commit(bar);
        }
        mma_pending = true;
        ok = mbar_wait(bar, phase);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        mma_pending = false;
        phase ^= 1;
        fence_after();
        epilogue_hidden(tm + lane_base + kLsHidden, sb + kLsHidden, Hs, t);
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int ks = 0; ks < kLsHidden / 16; ++ks)
                mma_bf16(tm, sdesc(a_h + ks * 2 * kLbo128, kLbo128, kSbo),
                         sdesc(a_w3 + ks * 2 * kLbo16, kLbo16, kSbo), id16, ks);
            mma_commit(bar);
        }
        mma_pending = true;
        ok = mbar_wait(bar, phase);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        mma_pending = false;
        phase ^= 1;
        fence_after();
        float o[16];
        tmem_ld16(tm + lane_base, o);
        const float4 *Sr = (const float4 *)(L.S[slot] + (size_t)row * 3 * kLsVec);
        float sv[3 * kLsVec];
#pragma unroll
        for (int q = 0; q < 3 * kLsVec / 4; ++q) {
            const float4 v = Sr[q];
            sv[4 * q] = v.x;
            sv[4 * q + 1] = v.y;
            sv[4 * q + 2] = v.z;
            sv[4 * q + 3] = v.w;
        }
        float gv[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int b = 0; b < kLsVec; ++b) {
            const float c = scale * (o[b] + sb[2 * kLsHidden + b]);
#pragma unroll
            for (int d = 0; d < 3; ++d) gv[d] = fmaf(c, sv[3 * b + d], gv[d]);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) L.G[slot][(size_t)d * n_rows + row] = gv[d];
        fence_before();  // accumulator reads before the next tile's MMAs
    }
    if (t == 0) {
        // a wait gave up: report, then let the MMAs and copies still in
        // flight finish (waits with the full limit) before the tensor memory
        // is freed and the CTA's shared memory released
        if (!ok) raise_status(status, MDG_ERR_TIMEOUT);
        if (mma_pending) mbar_wait(bar, phase);
        if (copy_pending) mbar_wait(tbar, tphase);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (w == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm),
                     "r"(kTmemCols)
                     : "memory");
}

// BF16 weight images in the tensor-core operand layout (B = W^T, N x K)
__global__ void __launch_bounds__(256) k_ls_tc_layout(Learned L) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    constexpr int n1 = kLsFeat * kLsHidden, n2 = kLsHidden * kLsHidden, n3 = kLsHidden * kLsVec;
    if (e >= n1 + n2 + n3) return;
    const uint16_t *src = L.wb;
    uint16_t *dst = L.wb + kLsWb;
    if (e < n1) {  // W1 [64][128] -> N = 128 rows (outputs), K = 64
        const int k = e / kLsHidden, nn = e % kLsHidden;
        dst[tc_off(nn, k, kLsHidden)] = src[e];
    } else if (e < n1 + n2) {  // W2 [128][128]
        const int q = e - n1, k = q / kLsHidden, nn = q % kLsHidden;
        dst[n1 + tc_off(nn, k, kLsHidden)] = src[e];
    } else {  // W3 [128][16] -> N = 16 rows, K = 128
        const int q = e - n1 - n2, k = q / kLsVec, nn = q % kLsVec;
        dst[n1 + n2 + tc_off(nn, k, kLsVec)] = src[e];
    }
}

}  // namespace

int ls_tc_prepare(mdg_system *) {
    if (cudaFuncSetAttribute(k_ls_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTcSmemAlloc) != cudaSuccess)
        return MDG_ERR_CUDA;
    return MDG_OK;
}

// slot < 0: lay out the weight images; else the forward pass of `slot`
cudaError_t ls_mlp_tc(mdg_system *s, int slot) {
    Learned &L = *s->ls;
    cudaStream_t st = s->stream;
    if (slot < 0) {
        k_ls_tc_layout<<<(kLsWb + 255) / 256, 256, 0, st>>>(L);
        s->launches += 1;
        return cudaGetLastError();
    }
    const int grid = std::min(L.n_tiles, 2 * std::max(1, s->n_sms));
    k_ls_mlp_tc<<<grid, kTcThreads, kTcSmemAlloc, st>>>(L, L.n_rows, slot, s->status);
    L.tc_wait_test = 0;  // one launch only
    s->launches += 1;
    return cudaGetLastError();
}

}  // namespace mdg
