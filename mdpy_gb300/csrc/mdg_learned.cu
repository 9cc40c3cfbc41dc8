// mdg_learned.cu -- learned slow force for the multiple-time-step form.
//
// The slow force of an evaluation is the reciprocal-space (PME) force plus
// the excluded-pair correction that removes the reciprocal sum's share of
// 1-2/1-3 pairs (the two vary slowly together; each alone follows the O-H
// vibration).  Full PME runs every k-th step.  In between, the slow force is
// predicted as
//     F_slow(t) ~ F_slow(t0) + G(x(t)) - G(x(t0))
// with t0 the last full evaluation and G a small rotation-equivariant
// network: per atom, 64 invariant features (32 cubic B-spline radial bins of
// the neighbours' charges and of their count, within rf), a BF16 MLP
// 64 -> 128 -> 128 -> 16 with SiLU and FP32 accumulation, whose 16 outputs
// are coefficients on the vectors S_ib = q_i sum_j q_j psi_b(r_ij) d_ij / rf^2
// (16 cubic B-spline radial functions psi_b, d_ij = x_i - x_j):
//     G_i = sum_b C_ib S_ib
// (optionally plus J_i (x_i(t) - x_i(t0)), the atom's motion through the
// field of the others).  Every k-th step the full PME result judges the
// prediction (relative RMS error against the total force); above the
// threshold the next interval falls back to the impulse scheme (the slow
// force enters at the interval's end with weight k), and the judge keeps
// running so the learned form resumes once its error is back under the
// threshold.
//
// Kernels (one system; atom order unless stated):
//   k_ls_pos       FP64 x -> wrapped FP32 positions; motion since the list
//                  was built (half the skin: rebuild)
//   k_ls_gate / k_ls_cells / k_ls_scan / k_ls_scatter / k_ls_cellsort
//                  atoms by cell of edge >= rf + skin, ascending index per cell
//   k_ls_list      neighbour list within rf + skin, 1-2/1-3 partners left
//                  out (a Verlet list: the build kernels run every step and
//                  return at once unless a rebuild is due)
//   k_ls_features  one thread per atom (cell order), bins accumulated in
//                  shared memory
//   k_ls_mlp       SIMT MLP (training forward, and the reference for the
//                  tensor-core kernel of mdg_learned_tc.cu)
//   k_ls_hessian / k_ls_hessian_excl
//                  optional field-gradient term J_i = d F_slow,i / d x_i
//   k_ls_apply     inner steps: f += F_slow(t0) - G(t0) + G(t) [+ J dx]
//   k_ls_judge     relative error of the prediction, mode of the next interval
//   k_ls_combine   slow force into f with the interval's weight; new base
//   training: k_ls_target, k_ls_residual, k_ls_dout, k_ls_backward,
//             k_ls_adam, k_ls_wb
// All sums that decide a trajectory run in a fixed order (neighbour lists in
// ascending atom order, per-block partials reduced in block order), so a run
// with given weights is bit-reproducible.
#include <cuda_bf16.h>

#include "mdg_internal.cuh"

namespace mdg {
namespace {

__device__ __forceinline__ float bf(uint16_t h) { return __uint_as_float((unsigned)h << 16); }
__device__ __forceinline__ uint16_t to_bf(float v) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }
// z sigmoid(z) (the tensor-core kernel uses the same expression)
__device__ __forceinline__ float silu(float z) {
    return __fdividef(z, 1.0f + __expf(-fmaxf(z, -80.0f)));
}
__device__ __forceinline__ float dsilu(float z) {
    const float s = sigm(z);
    return s * (1.0f + z * (1.0f - s));
}

// uniform cubic B-spline: weights of the bins i0-1 .. i0+2 at fraction t
__device__ __forceinline__ void bspline4(float t, float (&w)[4]) {
    const float t2 = t * t, t3 = t2 * t, u = 1.0f - t;
    w[0] = u * u * u * (1.0f / 6.0f);
    w[1] = (3.0f * t3 - 6.0f * t2 + 4.0f) * (1.0f / 6.0f);
    w[2] = (-3.0f * t3 + 3.0f * t2 + 3.0f * t + 1.0f) * (1.0f / 6.0f);
    w[3] = t3 * (1.0f / 6.0f);
}

struct Geo {
    int n, n_rows, n_pad;
    float L[3], invL[3], ncl[3];  // box, inverse, cells per A
    double Ld[3], invLd[3];
    float rf2, rl2, half_skin2, inv_h1, inv_h2, s_scale;
    // PME potential grid of the system (order 4) for the field-gradient term
    const float *phi;
    int K[3];
    float kl[3];
    float beta, self_h;  // Ewald beta; 4 beta^3 / (3 sqrt(pi))
};

// Wrapped FP32 positions of every atom; raises the rebuild flag when an
// atom has moved more than half the skin since the list was built.
__global__ void __launch_bounds__(256) k_ls_pos(const double *__restrict__ x,
                                                const float *__restrict__ q, Learned L, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool moved = false;
    if (i < g.n) {
        float p[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double c = x[3 * i + d];
            c -= g.Ld[d] * floor(c * g.invLd[d]);
            float v = (float)c;
            if (!(v >= 0.f) || v >= g.L[d]) v = 0.f;
            p[d] = v;
        }
        L.pos[i] = make_float4(p[0], p[1], p[2], q[i]);
        L.cpos[L.slot_of[i]] = make_float4(p[0], p[1], p[2], q[i]);
        const float4 r = L.xref[i];
        float d0 = p[0] - r.x, d1 = p[1] - r.y, d2 = p[2] - r.z;
        d0 -= g.L[0] * rintf(d0 * g.invL[0]);
        d1 -= g.L[1] * rintf(d1 * g.invL[1]);
        d2 -= g.L[2] * rintf(d2 * g.invL[2]);
        moved = d0 * d0 + d1 * d1 + d2 * d2 > g.half_skin2;
    }
    if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(&L.flag[0], 1);
}

// flag[1] = rebuild the list at this full evaluation (requested by motion,
// or forced); flag[0] starts collecting the next request
__global__ void k_ls_gate(Learned L, int force) {
    L.flag[1] = (L.flag[0] | force) ? 1 : 0;
    L.flag[0] = 0;
}

__global__ void __launch_bounds__(256) k_ls_cells(Learned L, Geo g) {
    if (!L.flag[1]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const float4 p = L.pos[i];
    const int c0 = min((int)(p.x * g.ncl[0]), L.nc[0] - 1);
    const int c1 = min((int)(p.y * g.ncl[1]), L.nc[1] - 1);
    const int c2 = min((int)(p.z * g.ncl[2]), L.nc[2] - 1);
    const int cell = (c0 * L.nc[1] + c1) * L.nc[2] + c2;
    L.cell_of[i] = cell;
    atomicAdd(&L.cell_count[cell], 1);
}

// cell starts (exclusive scan, start[n_cells] = n) from the counts, which it
// zeroes for the next build; resets the cursors.  One block.
__global__ void __launch_bounds__(1024) k_ls_scan(Learned L) {
    if (!L.flag[1]) return;
    __shared__ int s_w[32];
    const int n = L.n_cells, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (n + 1023) / 1024, lo = min(n, t * per), hi = min(n, lo + per);
    int sum = 0;
    for (int c = lo; c < hi; ++c) sum += L.cell_count[c];
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) s_w[w] = inc;
    __syncthreads();
    if (w == 0) {
        int v = s_w[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        s_w[lane] = v;
    }
    __syncthreads();
    int run = inc - sum + (w ? s_w[w - 1] : 0);
    for (int c = lo; c < hi; ++c) {
        L.cell_start[c] = run;
        run += L.cell_count[c];
        L.cell_count[c] = 0;
        L.cell_cursor[c] = 0;
    }
    if (t == 1023) L.cell_start[n] = run;
}

__global__ void __launch_bounds__(256) k_ls_scatter(Learned L, int n) {
    if (!L.flag[1]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = L.cell_of[i];
    L.cell_atoms[L.cell_start[c] + atomicAdd(&L.cell_cursor[c], 1)] = i;
}

// Ascending atom index within each cell (the scatter's order is arbitrary)
// and the cell-ordered copy of the positions.  One warp per cell: every
// element's rank is the number of smaller indices in the cell (indices are
// distinct); cells above 128 atoms sort on one lane.
__global__ void __launch_bounds__(256) k_ls_cellsort(Learned L) {
    if (!L.flag[1]) return;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (c >= L.n_cells) return;
    int *a = L.cell_atoms + L.cell_start[c];
    float4 *cp = L.cpos + L.cell_start[c];
    const int m = L.cell_start[c + 1] - L.cell_start[c];
    if (m <= 128) {
        int v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = lane + 32 * q < m ? a[lane + 32 * q] : 0x7fffffff;
        int rank[4] = {0, 0, 0, 0};
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) {
            if (32 * q2 >= m) break;  // warp-uniform
            for (int src = 0; src < 32; ++src) {
                const int o = __shfl_sync(0xffffffffu, v[q2], src);
#pragma unroll
                for (int q = 0; q < 4; ++q) rank[q] += o < v[q];
            }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (lane + 32 * q < m) {
                a[rank[q]] = v[q];
                cp[rank[q]] = L.pos[v[q]];
            }
        return;
    }
    if (lane == 0)
        for (int u = 1; u < m; ++u) {
            const int v = a[u];
            int w = u - 1;
            while (w >= 0 && a[w] > v) {
                a[w + 1] = a[w];
                --w;
            }
            a[w + 1] = v;
        }
    __syncwarp();
    for (int u = lane; u < m; u += 32) cp[u] = L.pos[a[u]];
}

// Neighbour list of slot s (cell order: a warp's atoms share most of their
// 27 cells, read from the cell-ordered positions), entries list[e][s] are
// slots too, so the feature kernel reads its neighbours from the
// cell-ordered copy that k_ls_pos refreshes every step.
// 1-2 / 1-3 partners (the reciprocal sum and the excluded-pair correction
// cancel for them, so they carry no slow force) are left out.  Stores the
// build positions for the motion test.
constexpr int kMaxPw = 8;

__global__ void __launch_bounds__(128) k_ls_list(Learned L, Geo g, const int *__restrict__ partners,
                                                 int pw, int *status) {
    if (!L.flag[1]) return;
    const int s0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (s0 >= g.n) return;
    const int i = L.cell_atoms[s0];
    const float4 pi = L.cpos[s0];
    L.xref[i] = pi;
    L.slot_of[i] = s0;
    int pr[kMaxPw];
#pragma unroll
    for (int u = 0; u < kMaxPw; ++u) pr[u] = u < pw ? partners[(size_t)i * pw + u] : -1;
    const int c = L.cell_of[i];
    const int cz = c % L.nc[2], cy = (c / L.nc[2]) % L.nc[1], cx = c / (L.nc[1] * L.nc[2]);
    int cnt = 0;
    for (int dx = -1; dx <= 1; ++dx) {
        const int x1 = (cx + dx + L.nc[0]) % L.nc[0];
        for (int dy = -1; dy <= 1; ++dy) {
            const int y1 = (cy + dy + L.nc[1]) % L.nc[1];
            for (int dz = -1; dz <= 1; ++dz) {
                const int z1 = (cz + dz + L.nc[2]) % L.nc[2];
                const int cell = (x1 * L.nc[1] + y1) * L.nc[2] + z1;
                const int st = L.cell_start[cell], en = L.cell_start[cell + 1];
#pragma unroll 4
                for (int q = st; q < en; ++q) {
                    const float4 pj = __ldg(&L.cpos[q]);
                    float d0 = pi.x - pj.x, d1 = pi.y - pj.y, d2 = pi.z - pj.z;
                    d0 -= g.L[0] * rintf(d0 * g.invL[0]);
                    d1 -= g.L[1] * rintf(d1 * g.invL[1]);
                    d2 -= g.L[2] * rintf(d2 * g.invL[2]);
                    if (d0 * d0 + d1 * d1 + d2 * d2 >= g.rl2) continue;
                    const int j = __ldg(&L.cell_atoms[q]);
                    if (j == i) continue;
                    bool excluded = false;
#pragma unroll
                    for (int u = 0; u < kMaxPw; ++u) excluded |= pr[u] == j;
                    for (int u = kMaxPw; u < pw; ++u) excluded |= partners[(size_t)i * pw + u] == j;
                    if (excluded) continue;
                    if (cnt < L.cap) L.list[(size_t)cnt * g.n + s0] = q;
                    ++cnt;
                }
            }
        }
    }
    L.nlist[s0] = min(cnt, L.cap);
    if (cnt > L.cap) raise_status(status, MDG_ERR_OVERFLOW);
}

// Features and vector basis, one thread per slot of the list.  A thread's
// 132 FP32 accumulators are column t of a [132][64] shared array (every
// access conflict free); the bins carry one padding bin below and two above
// so that a pair's four B-spline weights always land in valid slots, and
// each pair loads its 20 accumulators, adds, and stores them back (all 20
// distinct).  The next entry's index and position load one step ahead.
// Sums run in list order: the result does not depend on scheduling.
constexpr int kFeatThreads = 64;
constexpr int kFB = kLsBins + 4;            // padded feature bins (b = -1 .. 34)
constexpr int kVB = kLsVec + 4;             // padded vector bins
constexpr int kAccP = 2 * kFB + 3 * kVB;    // 72 + 60

template <bool RAW>
__global__ void __launch_bounds__(kFeatThreads) k_ls_features(Learned L, Geo g, int slot,
                                                             int gated) {
    __shared__ float acc[kAccP * kFeatThreads];
    if (gated && *L.mode != kLsLearned) return;
    const int t = threadIdx.x, s0 = blockIdx.x * kFeatThreads + t;
    float *a = acc + t;
#pragma unroll 4
    for (int b = 0; b < kAccP; ++b) a[b * kFeatThreads] = 0.f;
    if (s0 >= g.n) return;  // no block barrier in this kernel
    const int i = L.cell_atoms[s0];
    const float4 pi = L.cpos[s0];
    const int cnt = L.nlist[s0];
    constexpr int kB = 8;  // entries whose loads are in flight together
    for (int e0 = 0; e0 < cnt; e0 += kB) {
        float4 pb[kB];
#pragma unroll
        for (int m = 0; m < kB; ++m) {
            const int jj = e0 + m < cnt ? __ldg(&L.list[(size_t)(e0 + m) * g.n + s0]) : s0;
            pb[m] = __ldg(&L.cpos[jj]);
        }
#pragma unroll
        for (int m = 0; m < kB; ++m) {
        if (e0 + m >= cnt) break;
        const float4 pc = pb[m];
        float d0 = pi.x - pc.x, d1 = pi.y - pc.y, d2 = pi.z - pc.z;
        d0 -= g.L[0] * rintf(d0 * g.invL[0]);
        d1 -= g.L[1] * rintf(d1 * g.invL[1]);
        d2 -= g.L[2] * rintf(d2 * g.invL[2]);
        const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
        if (!(r2 < g.rf2) || r2 == 0.f) continue;
        const float r = sqrtf(r2);
        float w1[4], w2[4];
        const float u1 = r * g.inv_h1, u2 = r * g.inv_h2;
        const int i1 = min((int)u1, kLsBins), i2 = min((int)u2, kLsVec);
        bspline4(u1 - (float)i1, w1);
        bspline4(u2 - (float)i2, w2);
        // padded slot of bin b = i - 1 + m is i + m
        float *fq = a + i1 * kFeatThreads, *fc = a + (kFB + i1) * kFeatThreads;
        float *fv = a + (2 * kFB + 3 * i2) * kFeatThreads;
        float vq[4], vc[4], vv[12];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            vq[m] = fq[m * kFeatThreads];
            vc[m] = fc[m * kFeatThreads];
        }
#pragma unroll
        for (int m = 0; m < 12; ++m) vv[m] = fv[m * kFeatThreads];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            vq[m] = fmaf(pc.w, w1[m], vq[m]);
            vc[m] += w1[m];
            const float c = pc.w * w2[m];
            vv[3 * m] = fmaf(c, d0, vv[3 * m]);
            vv[3 * m + 1] = fmaf(c, d1, vv[3 * m + 1]);
            vv[3 * m + 2] = fmaf(c, d2, vv[3 * m + 2]);
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            fq[m * kFeatThreads] = vq[m];
            fc[m * kFeatThreads] = vc[m];
        }
#pragma unroll
        for (int m = 0; m < 12; ++m) fv[m * kFeatThreads] = vv[m];
        }
    }
    // features (bins 0..31 sit in padded slots 1..32): normalised, BF16, tile
    // layout, 8 features (one 16-byte core-matrix row) per store
#pragma unroll 1
    for (int k0 = 0; k0 < kLsFeat; k0 += 8) {
        unsigned h[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int k = k0 + 2 * u;
            const int p0 = (k < kLsBins ? k : kFB + k - kLsBins) + 1;
            const float r0 = a[p0 * kFeatThreads], r1 = a[(p0 + 1) * kFeatThreads];
            if (RAW) *(float2 *)(L.xraw[slot] + (size_t)i * kLsFeat + k) = make_float2(r0, r1);
            const float n0 = (r0 - L.params[kLsMu + k]) * L.params[kLsSig + k];
            const float n1 = (r1 - L.params[kLsMu + k + 1]) * L.params[kLsSig + k + 1];
            h[u] = (unsigned)to_bf(n0) | ((unsigned)to_bf(n1) << 16);
        }
        *(uint4 *)(L.xb[slot] + ls_xoff(i, k0)) = make_uint4(h[0], h[1], h[2], h[3]);
    }
    const float qs = pi.w * g.s_scale;
    float4 *so = (float4 *)(L.S[slot] + (size_t)i * 3 * kLsVec);
#pragma unroll 4
    for (int c = 0; c < 3 * kLsVec; c += 4)
        so[c / 4] = make_float4(a[(2 * kFB + 3 + c) * kFeatThreads] * qs,
                                a[(2 * kFB + 4 + c) * kFeatThreads] * qs,
                                a[(2 * kFB + 5 + c) * kFeatThreads] * qs,
                                a[(2 * kFB + 6 + c) * kFeatThreads] * qs);
}

// ---- SIMT MLP ---------------------------------------------------------------
constexpr int kH2Stride = kLsHidden + 2;  // conflict-free row reads in layer 3

template <int TM, int TN, class FA, class FB>
__device__ __forceinline__ void mm_acc(float (&acc)[TM][TN], int K, FA fa, FB fb) {
#pragma unroll 2
    for (int k = 0; k < K; ++k) {
        float av[TM], bv[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) av[i] = fa(i, k);
#pragma unroll
        for (int j = 0; j < TN; ++j) bv[j] = fb(k, j);
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
}

__device__ __forceinline__ void copy16(void *dst, const void *src, int bytes) {
    const uint4 *s = (const uint4 *)src;
    uint4 *d = (uint4 *)dst;
    for (int e = threadIdx.x; e < bytes / 16; e += blockDim.x) d[e] = s[e];
}

constexpr size_t kMlpSmem =
    sizeof(uint16_t) * (kLsTile * kLsFeat + kLsFeat * kLsHidden + kLsTile * kLsHidden +
                        kLsHidden * kLsHidden + kLsHidden * kLsVec + kLsTile * kH2Stride) +
    sizeof(float) * (2 * kLsHidden + kLsVec);

// One 128-atom tile per CTA of 256 threads; layers 1 and 2 give each thread an
// 8 x 8 block of the tile's outputs.  TRAIN keeps the pre-activations.
template <bool TRAIN>
__global__ void __launch_bounds__(256) k_ls_mlp(Learned L, Geo g, int slot) {
    extern __shared__ __align__(16) unsigned char smraw[];
    uint16_t *Xs = (uint16_t *)smraw;
    uint16_t *W1s = Xs + kLsTile * kLsFeat;
    uint16_t *H1s = W1s + kLsFeat * kLsHidden;
    uint16_t *W2s = H1s + kLsTile * kLsHidden;
    uint16_t *W3s = W2s + kLsHidden * kLsHidden;
    uint16_t *H2s = W3s + kLsHidden * kLsVec;
    float *sb = (float *)(H2s + kLsTile * kH2Stride);
    const int t = threadIdx.x, row0 = blockIdx.x * kLsTile;
    copy16(Xs, L.xb[slot] + (size_t)row0 * kLsFeat, 2 * kLsTile * kLsFeat);
    copy16(W1s, L.wb, 2 * kLsFeat * kLsHidden);
    copy16(W2s, L.wb + kLsFeat * kLsHidden, 2 * kLsHidden * kLsHidden);
    copy16(W3s, L.wb + kLsFeat * kLsHidden + kLsHidden * kLsHidden, 2 * kLsHidden * kLsVec);
    for (int e = t; e < kLsHidden; e += 256) {
        sb[e] = L.params[kLsB1 + e];
        sb[kLsHidden + e] = L.params[kLsB2 + e];
    }
    if (t < kLsVec) sb[2 * kLsHidden + t] = L.params[kLsB3 + t];
    __syncthreads();
    const int rg = t >> 4, cg = t & 15;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = sb[cg * 8 + j];
    mm_acc(acc, kLsFeat, [&](int i, int k) { return bf(Xs[ls_tc_off(rg * 8 + i, k, kLsTile)]); },
           [&](int k, int j) { return bf(W1s[k * kLsHidden + cg * 8 + j]); });
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int r = rg * 8 + i, c = cg * 8 + j;
            if (TRAIN) L.Z1[slot][(size_t)(row0 + r) * kLsHidden + c] = acc[i][j];
            H1s[r * kLsHidden + c] = to_bf(silu(acc[i][j]));
        }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = sb[kLsHidden + cg * 8 + j];
    mm_acc(acc, kLsHidden, [&](int i, int k) { return bf(H1s[(rg * 8 + i) * kLsHidden + k]); },
           [&](int k, int j) { return bf(W2s[k * kLsHidden + cg * 8 + j]); });
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int r = rg * 8 + i, c = cg * 8 + j;
            if (TRAIN) L.Z2[slot][(size_t)(row0 + r) * kLsHidden + c] = acc[i][j];
            H2s[r * kH2Stride + c] = to_bf(silu(acc[i][j]));
        }
    __syncthreads();
    // layer 3 and the force: thread = (row, half of the 16 outputs)
    const int row = t & (kLsTile - 1), half = t >> 7;
    float o[1][8];
#pragma unroll
    for (int j = 0; j < 8; ++j) o[0][j] = sb[2 * kLsHidden + half * 8 + j];
    mm_acc(o, kLsHidden, [&](int, int k) { return bf(H2s[row * kH2Stride + k]); },
           [&](int k, int j) { return bf(W3s[k * kLsVec + half * 8 + j]); });
    const float sc = L.params[kLsScale];
    const int gr = row0 + row;
    float gv[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int b = half * 8 + j;
        const float c = sc * o[0][j];
#pragma unroll
        for (int d = 0; d < 3; ++d) gv[d] = fmaf(c, L.S[slot][(size_t)gr * 3 * kLsVec + 3 * b + d], gv[d]);
    }
    // the two halves of a row sit 128 threads apart: combine through shared memory
    __syncthreads();
    float *red = (float *)Xs;  // Xs is free after layer 1
    if (half == 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) red[3 * row + d] = gv[d];
    }
    __syncthreads();
    if (half == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            gv[d] += red[3 * row + d];
            L.G[slot][(size_t)d * g.n_rows + gr] = gv[d];
        }
    }
}

// Sums n pairs of per-block partials (red[2u], red[2u+1]) in a fixed order
// with the 256 threads of a block: strided partial sums, then a fixed tree.
__device__ void reduce_pairs(const double *red, int n, double &a, double &b) {
    __shared__ double s_a[256], s_b[256];
    double x = 0.0, y = 0.0;
    for (int u = threadIdx.x; u < n; u += 256) {
        x += ((const volatile double *)red)[2 * u];
        y += ((const volatile double *)red)[2 * u + 1];
    }
    s_a[threadIdx.x] = x;
    s_b[threadIdx.x] = y;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            s_a[threadIdx.x] += s_a[threadIdx.x + h];
            s_b[threadIdx.x] += s_b[threadIdx.x + h];
        }
        __syncthreads();
    }
    a = s_a[0];
    b = s_b[0];
    __syncthreads();
}

// ---- field-gradient (Taylor) term -------------------------------------------
// J_i = d F_slow,i / d x_i with the other atoms held: -q_i times the Hessian
// of the reciprocal potential at x_i (order-4 B-spline second derivatives of
// the PME potential grid), less the atom's own smeared charge (a constant
// -4 beta^3 / (3 sqrt pi) q_i^2 I in J) and less its excluded partners (added
// back pair by pair below: their share cancels against the excluded-pair
// correction).  Then F_slow,i(t) ~ F_slow,i(t0) + J_i (x_i(t) - x_i(t0)).
__device__ __forceinline__ void bspline4_d2(float w, float (&th)[4], float (&dth)[4],
                                            float (&ddth)[4]) {
    // grid point g0 + c carries M4(w + 3 - c) (the PME kernels' indexing)
    const float w2 = w * w, w3 = w2 * w, u = 1.f - w;
    th[0] = u * u * u * (1.f / 6.f);
    th[1] = (3.f * w3 - 6.f * w2 + 4.f) * (1.f / 6.f);
    th[2] = (-3.f * w3 + 3.f * w2 + 3.f * w + 1.f) * (1.f / 6.f);
    th[3] = w3 * (1.f / 6.f);
    dth[0] = -0.5f * u * u;
    dth[1] = 1.5f * w2 - 2.f * w;
    dth[2] = -1.5f * w2 + w + 0.5f;
    dth[3] = 0.5f * w2;
    ddth[0] = u;
    ddth[1] = 3.f * w - 2.f;
    ddth[2] = 1.f - 3.f * w;
    ddth[3] = w;
}

__global__ void __launch_bounds__(256) k_ls_hessian(Learned L, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const float4 p = L.pos[i];
    float th[3][4], dth[3][4], ddth[3][4];
    int g0[3];
    const float xs[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int K = g.K[d];
        float u = fmodf(xs[d] * g.kl[d], (float)K);
        if (u < 0.f) u += (float)K;
        if (!(u >= 0.f && u < (float)K)) u = 0.f;
        int m = min((int)u, K - 1);
        const float w = u - (float)m;
        g0[d] = m - 3;
        if (g0[d] < 0) g0[d] += K;
        bspline4_d2(w, th[d], dth[d], ddth[d]);
    }
    float h[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // xx yy zz xy xz yz
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int ga = (g0[0] + a) % g.K[0];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gb = (g0[1] + b) % g.K[1];
            const float *row = g.phi + ((size_t)ga * g.K[1] + gb) * g.K[2];
            float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float v = __ldg(&row[(g0[2] + c) % g.K[2]]);
                s0 = fmaf(th[2][c], v, s0);
                s1 = fmaf(dth[2][c], v, s1);
                s2 = fmaf(ddth[2][c], v, s2);
            }
            h[0] = fmaf(ddth[0][a] * th[1][b], s0, h[0]);
            h[1] = fmaf(th[0][a] * ddth[1][b], s0, h[1]);
            h[2] = fmaf(th[0][a] * th[1][b], s2, h[2]);
            h[3] = fmaf(dth[0][a] * dth[1][b], s0, h[3]);
            h[4] = fmaf(dth[0][a] * th[1][b], s1, h[4]);
            h[5] = fmaf(th[0][a] * dth[1][b], s1, h[5]);
        }
    }
    const float q = p.w, sh = g.self_h * q * q;
    const float sc[6] = {g.kl[0] * g.kl[0], g.kl[1] * g.kl[1], g.kl[2] * g.kl[2],
                         g.kl[0] * g.kl[1], g.kl[0] * g.kl[2], g.kl[1] * g.kl[2]};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const float jv = -q * h[c] * sc[c] - (c < 3 ? sh : 0.f);
        L.Jn[(size_t)c * g.n + i] = to_fix(jv);
    }
}

// + q_i q_j Hess k(r_ij), k(r) = erf(beta r) / r, for each excluded pair
__global__ void __launch_bounds__(256) k_ls_hessian_excl(Learned L, Geo g,
                                                         const int2 *__restrict__ excl, int n_excl) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_excl) return;
    const int2 pr = excl[t];
    const float4 pi = L.pos[pr.x], pj = L.pos[pr.y];
    float d[3] = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] -= g.L[k] * rintf(d[k] * g.invL[k]);
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (!(r2 > 0.f)) return;
    const float r = sqrtf(r2), br = g.beta * r;
    const float ef = erff(br);
    const float gg = 1.1283791670955126f * g.beta * expf(-br * br);  // 2 beta / sqrt(pi) e^-b2r2
    const float k1 = gg / r - ef / r2;                                 // k'
    const float k2 = -2.f * g.beta * g.beta * gg - 2.f * gg / r2 + 2.f * ef / (r2 * r);  // k''
    const float qq = pi.w * pj.w;
    const float a = qq * (k2 - k1 / r) / r2, b = qq * k1 / r;  // H = a d d^T + b I
    const float hv[6] = {a * d[0] * d[0] + b, a * d[1] * d[1] + b, a * d[2] * d[2] + b,
                         a * d[0] * d[1], a * d[0] * d[2], a * d[1] * d[2]};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const long long v = to_fix(hv[c]);
        fix_red((unsigned long long *)&L.Jn[(size_t)c * g.n + pr.x], v);
        fix_red((unsigned long long *)&L.Jn[(size_t)c * g.n + pr.y], v);
    }
}

// J (x - x0) with the minimum image, from a fixed-point J
__device__ __forceinline__ void taylor_term(const long long *J, int n, int i, float4 x, float4 x0,
                                            const Geo &g, float (&out)[3]) {
    float d[3] = {x.x - x0.x, x.y - x0.y, x.z - x0.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] -= g.L[k] * rintf(d[k] * g.invL[k]);
    float j[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) j[c] = (float)((double)J[(size_t)c * n + i] * kFixInv);
    out[0] = j[0] * d[0] + j[3] * d[1] + j[4] * d[2];
    out[1] = j[3] * d[0] + j[1] * d[1] + j[5] * d[2];
    out[2] = j[4] * d[0] + j[5] * d[1] + j[2] * d[2];
}

// inner step of the learned form: f += base + G + J (x - x0)
__global__ void __launch_bounds__(256) k_ls_apply(Learned L, Geo g, const int *__restrict__ inv_perm,
                                                  unsigned long long *__restrict__ f, int taylor,
                                                  int net) {
    if (*L.mode != kLsLearned) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    float tt[3] = {0.f, 0.f, 0.f};
    if (taylor) taylor_term(L.J, g.n, i, L.pos[i], L.x0[i], g, tt);
    const int k = inv_perm[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        long long v = L.base[(size_t)d * g.n + i] + to_fix(tt[d]);
        if (net) v += to_fix(L.G[0][(size_t)d * g.n_rows + i]);
        fix_red(&f[(size_t)d * g.n_pad + k], v);
    }
}

// ---- judge and combine (outer steps) ----------------------------------------
// Relative RMS error of the prediction base + G against the slow force just
// computed, normalised by the total force; the last block reduces the
// per-block partials in block order and sets the mode of the next interval.
__global__ void __launch_bounds__(256) k_ls_judge(Learned L, Geo g, const int *__restrict__ inv_perm,
                                                  const unsigned long long *__restrict__ f,
                                                  int anchor, int *done, int taylor, int net) {
    __shared__ double s_e[8], s_t[8];
    __shared__ bool last;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e2 = 0.0, t2 = 0.0;
    if (i < g.n && !anchor) {
        const int k = inv_perm[i];
        float tt[3] = {0.f, 0.f, 0.f};
        if (taylor) taylor_term(L.J, g.n, i, L.pos[i], L.x0[i], g, tt);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const long long fs = (long long)L.fs[(size_t)d * g.n_pad + k];
            long long pr = L.base[(size_t)d * g.n + i] + to_fix(tt[d]);
            if (net) pr += to_fix(L.G[0][(size_t)d * g.n_rows + i]);
            const double e = (double)(pr - fs) * kFixInv;
            const double tt = (double)((long long)f[(size_t)d * g.n_pad + k] + fs) * kFixInv;
            e2 += e * e;
            t2 += tt * tt;
        }
    }
    e2 = warp_sum_d(e2);
    t2 = warp_sum_d(t2);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_e[w] = e2;
        s_t[w] = t2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int u = 0; u < 8; ++u) {
            a += s_e[u];
            b += s_t[u];
        }
        L.red[2 * blockIdx.x] = a;
        L.red[2 * blockIdx.x + 1] = b;
        __threadfence();
        last = atomicAdd(done, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0, b = 0.0;
    reduce_pairs(L.red, (int)gridDim.x, a, b);
    if (threadIdx.x != 0) return;
    *done = 0;
    L.mode[1] = L.mode[0];  // the interval that just ended
    if (anchor) {
        L.mode[0] = kLsLearned;
        L.mode[1] = kLsLearned;
        return;
    }
    const double err = b > 0.0 ? sqrt(a / b) : 0.0;
    L.stats[0] = err;
    L.stats[1] = fmax(L.stats[1], err);
    L.stats[2] += err;
    L.stats[3] += 1.0;
    const int next = err > (double)L.threshold ? kLsImpulse : kLsLearned;
    if (next == kLsImpulse) L.stats[4] += 1.0;
    L.mode[0] = next;
}

// f += w F_slow with w the mean of the weights of the intervals either side
// (learned 1, impulse k): the two half kicks that use this force then give
// the slow force its exact total weight; base = F_slow - G for the interval
// that starts here.
__global__ void __launch_bounds__(256) k_ls_combine(Learned L, Geo g, const int *__restrict__ inv_perm,
                                                    unsigned long long *__restrict__ f, int kout,
                                                    int net) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const long long w2 = (L.mode[0] == kLsLearned ? 1 : kout) + (L.mode[1] == kLsLearned ? 1 : kout);
    const int k = inv_perm[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long fs = (long long)L.fs[(size_t)d * g.n_pad + k];
        // w2 is even unless one side is learned and k is even: then the
        // half-integer weight rounds the fixed-point word to nearest
        const long long add = (w2 & 1) ? (fs * w2 + (fs >= 0 ? 1 : -1)) / 2 : fs * (w2 / 2);
        f[(size_t)d * g.n_pad + k] += (unsigned long long)add;
        L.base[(size_t)d * g.n + i] = fs - (net ? to_fix(L.G[0][(size_t)d * g.n_rows + i]) : 0ll);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) L.J[(size_t)c * g.n + i] = L.Jn[(size_t)c * g.n + i];
    L.x0[i] = L.pos[i];
}

// ---- training -----------------------------------------------------------------
// slow-force target of a frame, atom order, float
__global__ void __launch_bounds__(256) k_ls_target(Learned L, Geo g, const int *__restrict__ inv_perm,
                                                   int slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    L.fpos[slot][i] = L.pos[i];
    if (slot == 0)  // the field-gradient term of the pair's first frame
#pragma unroll
        for (int c = 0; c < 6; ++c) L.J[(size_t)c * g.n + i] = L.Jn[(size_t)c * g.n + i];
    const int k = inv_perm[i];
#pragma unroll
    for (int d = 0; d < 3; ++d)
        L.T[slot][(size_t)d * g.n + i] =
            (float)((double)(long long)L.fs[(size_t)d * g.n_pad + k] * kFixInv);
}

// the network's target is the slow-force change less the field-gradient
// term (when that term is in use)
__device__ __forceinline__ void residual(const Learned &L, const Geo &g, int i, float (&R)[3],
                                         float (&dT)[3]) {
    float tt[3] = {0.f, 0.f, 0.f};
    if (L.use_taylor) taylor_term(L.J, g.n, i, L.fpos[1][i], L.fpos[0][i], g, tt);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dT[d] = L.T[1][(size_t)d * g.n + i] - L.T[0][(size_t)d * g.n + i] - tt[d];
        R[d] = (L.G[1][(size_t)d * g.n_rows + i] - L.G[0][(size_t)d * g.n_rows + i]) - dT[d];
    }
}

// per-block partials of sum |R|^2 and sum |dT|^2
__global__ void __launch_bounds__(256) k_ls_residual(Learned L, Geo g) {
    __shared__ double s_a[8], s_b[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, b = 0.0;
    if (i < g.n) {
        float R[3], dT[3];
        residual(L, g, i, R, dT);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a += (double)R[d] * R[d];
            b += (double)dT[d] * dT[d];
        }
    }
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    if ((threadIdx.x & 31) == 0) {
        s_a[threadIdx.x >> 5] = a;
        s_b[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int u = 0; u < 8; ++u) {
            x += s_a[u];
            y += s_b[u];
        }
        L.red[2 * blockIdx.x] = x;
        L.red[2 * blockIdx.x + 1] = y;
    }
}

// loss = sum |R|^2 / sum |dT|^2 (1 = no better than holding the slow force);
// gradients at the MLP outputs of both frames
__global__ void __launch_bounds__(256) k_ls_dout(Learned L, Geo g, int n_blocks) {
    __shared__ double s_tot[2];
    double a = 0.0, b = 0.0;
    reduce_pairs(L.red, n_blocks, a, b);
    if (threadIdx.x == 0) {
        s_tot[0] = a;
        s_tot[1] = b;
        if (blockIdx.x == 0) {
            L.stats[5] = b > 0.0 ? a / b : 0.0;
            L.stats[6] = b;
        }
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n_rows) return;
    float R[3] = {0.f, 0.f, 0.f}, dT[3];
    if (i < g.n) residual(L, g, i, R, dT);
    const float c = s_tot[1] > 0.0 ? (float)(2.0 / s_tot[1]) * L.params[kLsScale] : 0.f;
    for (int s = 0; s < 2; ++s) {
        const float sg = s ? c : -c;
#pragma unroll 4
        for (int b = 0; b < kLsVec; ++b) {
            float v = 0.f;
#pragma unroll
            for (int d = 0; d < 3; ++d) v = fmaf(R[d], L.S[s][(size_t)i * 3 * kLsVec + 3 * b + d], v);
            L.dout[((size_t)s * g.n_rows + i) * kLsVec + b] = sg * v;
        }
    }
}

constexpr int kAStride = kLsHidden + 2;
constexpr size_t kBwdSmem = sizeof(float) * (2 * kLsTile * kLsHidden + kLsTile * kLsVec) +
                            sizeof(uint16_t) * (kLsTile * kAStride + kLsHidden * kLsHidden +
                                                kLsVec * kLsHidden);

// Backward through the MLP for (frame, tile) jobs; each CTA adds its jobs'
// weight gradients, in job order, to its own row of gpart (no atomics).
__global__ void __launch_bounds__(256) k_ls_backward(Learned L, Geo g) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float *dZ2 = (float *)smraw;
    float *dZ1 = dZ2 + kLsTile * kLsHidden;
    float *dO = dZ1 + kLsTile * kLsHidden;
    uint16_t *A = (uint16_t *)(dO + kLsTile * kLsVec);
    uint16_t *W2T = A + kLsTile * kAStride;
    uint16_t *W3T = W2T + kLsHidden * kLsHidden;
    const int t = threadIdx.x;
    const uint16_t *W1 = L.wb, *W2 = W1 + kLsFeat * kLsHidden, *W3 = W2 + kLsHidden * kLsHidden;
    (void)W1;
    for (int e = t; e < kLsHidden * kLsHidden; e += 256) {
        const int i = e >> 7, o = e & 127;
        W2T[o * kLsHidden + i] = W2[e];
    }
    for (int e = t; e < kLsHidden * kLsVec; e += 256) {
        const int h = e / kLsVec, b = e % kLsVec;
        W3T[b * kLsHidden + h] = W3[e];
    }
    float *gp = L.gpart + (size_t)blockIdx.x * kLsParams;
    const int rg = t >> 4, cg = t & 15;
    for (int job = blockIdx.x; job < 2 * g.n_rows / kLsTile; job += gridDim.x) {
        const int n_tiles = g.n_rows / kLsTile;
        const int slot = job / n_tiles, row0 = (job % n_tiles) * kLsTile;
        const float *Z1 = L.Z1[slot] + (size_t)row0 * kLsHidden;
        const float *Z2 = L.Z2[slot] + (size_t)row0 * kLsHidden;
        __syncthreads();
        for (int e = t; e < kLsTile * kLsVec; e += 256)
            dO[e] = L.dout[((size_t)slot * g.n_rows + row0) * kLsVec + e];
        for (int e = t; e < kLsTile * kLsHidden; e += 256)
            A[(e >> 7) * kAStride + (e & 127)] = to_bf(silu(Z2[e]));
        __syncthreads();
        {  // dW3 += H2^T dO, db3
            const int h = t >> 1, b0 = (t & 1) * 8;
            float acc[1][8] = {};
            mm_acc(acc, kLsTile, [&](int, int r) { return bf(A[r * kAStride + h]); },
                   [&](int r, int j) { return dO[r * kLsVec + b0 + j]; });
#pragma unroll
            for (int j = 0; j < 8; ++j) gp[kLsW3 + h * kLsVec + b0 + j] += acc[0][j];
            if (t < kLsVec) {
                float s = 0.f;
                for (int r = 0; r < kLsTile; ++r) s += dO[r * kLsVec + t];
                gp[kLsB3 + t] += s;
            }
        }
        {  // dZ2 = (dO W3^T) * silu'(Z2)
            float acc[8][8] = {};
            mm_acc(acc, kLsVec, [&](int i, int b) { return dO[(rg * 8 + i) * kLsVec + b]; },
                   [&](int b, int j) { return bf(W3T[b * kLsHidden + cg * 8 + j]); });
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int r = rg * 8 + i, c = cg * 8 + j;
                    dZ2[r * kLsHidden + c] = acc[i][j] * dsilu(Z2[r * kLsHidden + c]);
                }
        }
        __syncthreads();
        for (int e = t; e < kLsTile * kLsHidden; e += 256)
            A[(e >> 7) * kAStride + (e & 127)] = to_bf(silu(Z1[e]));
        __syncthreads();
        {  // dW2 += H1^T dZ2, db2
            float acc[8][8] = {};
            mm_acc(acc, kLsTile, [&](int i, int r) { return bf(A[r * kAStride + rg * 8 + i]); },
                   [&](int r, int j) { return dZ2[r * kLsHidden + cg * 8 + j]; });
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    gp[kLsW2 + (rg * 8 + i) * kLsHidden + cg * 8 + j] += acc[i][j];
            if (t < kLsHidden) {
                float s = 0.f;
                for (int r = 0; r < kLsTile; ++r) s += dZ2[r * kLsHidden + t];
                gp[kLsB2 + t] += s;
            }
        }
        {  // dZ1 = (dZ2 W2^T) * silu'(Z1)
            float acc[8][8] = {};
            mm_acc(acc, kLsHidden, [&](int i, int h) { return dZ2[(rg * 8 + i) * kLsHidden + h]; },
                   [&](int h, int j) { return bf(W2T[h * kLsHidden + cg * 8 + j]); });
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int r = rg * 8 + i, c = cg * 8 + j;
                    dZ1[r * kLsHidden + c] = acc[i][j] * dsilu(Z1[r * kLsHidden + c]);
                }
        }
        __syncthreads();
        {  // features into A, then dW1 += X^T dZ1, db1
            const uint16_t *X = L.xb[slot] + (size_t)row0 * kLsFeat;
            for (int e = t; e < kLsTile * kLsFeat; e += 256)
                A[(e >> 6) * kAStride + (e & 63)] = X[ls_tc_off(e >> 6, e & 63, kLsTile)];
        }
        __syncthreads();
        {
            const int kg = t >> 4, hg = t & 15;
            float acc[4][8] = {};
            mm_acc(acc, kLsTile, [&](int i, int r) { return bf(A[r * kAStride + kg * 4 + i]); },
                   [&](int r, int j) { return dZ1[r * kLsHidden + hg * 8 + j]; });
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    gp[kLsW1 + (kg * 4 + i) * kLsHidden + hg * 8 + j] += acc[i][j];
            if (t < kLsHidden) {
                float s = 0.f;
                for (int r = 0; r < kLsTile; ++r) s += dZ1[r * kLsHidden + t];
                gp[kLsB1 + t] += s;
            }
        }
    }
}

// Adam on the FP32 master (the feature normalisation and the output scale
// are fixed); sums the CTA partials in CTA order
__global__ void __launch_bounds__(256) k_ls_adam(Learned L, int n_parts, float lr_t, float b1,
                                                 float b2, float eps) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kLsParams || p < kLsW1 || p == kLsScale) return;
    float gsum = 0.f;
    for (int c = 0; c < n_parts; ++c) gsum += L.gpart[(size_t)c * kLsParams + p];
    const float m = b1 * L.adam_m[p] + (1.f - b1) * gsum;
    const float v = b2 * L.adam_v[p] + (1.f - b2) * gsum * gsum;
    L.adam_m[p] = m;
    L.adam_v[p] = v;
    L.params[p] -= lr_t * m / (sqrtf(v) + eps);
}

// BF16 copies of the three weight matrices ([in][out], concatenated)
__global__ void __launch_bounds__(256) k_ls_wb(Learned L) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kLsWb) return;
    constexpr int n1 = kLsFeat * kLsHidden, n2 = kLsHidden * kLsHidden;
    const int p = e < n1 ? kLsW1 + e : e < n1 + n2 ? kLsW2 + (e - n1) : kLsW3 + (e - n1 - n2);
    L.wb[e] = to_bf(L.params[p]);
}

Geo make_geo(const mdg_system *s) {
    const Learned &L = *s->ls;
    const SysDev &d = s->sys_h[0];
    Geo g;
    g.n = s->n;
    g.n_rows = L.n_rows;
    g.n_pad = s->n_pad;
    for (int k = 0; k < 3; ++k) {
        g.L[k] = d.L[k];
        g.invL[k] = d.invL[k];
        g.Ld[k] = d.Ld[k];
        g.invLd[k] = d.invLd[k];
        g.ncl[k] = (float)(L.nc[k] / d.Ld[k]);
    }
    g.rf2 = L.rf * L.rf;
    const float rl = L.rf + L.skin;
    g.rl2 = rl * rl;
    g.half_skin2 = 0.25f * L.skin * L.skin;
    g.phi = s->pme.grid_r ? s->pme.grid_r + d.grid_off : nullptr;
    for (int k = 0; k < 3; ++k) {
        g.K[k] = d.K[k];
        g.kl[k] = d.kl[k];
    }
    g.beta = (float)s->beta;
    g.self_h = (float)(4.0 * s->beta * s->beta * s->beta / (3.0 * 1.7724538509055159));
    g.inv_h1 = (float)(kLsBins + 1) / L.rf;
    g.inv_h2 = (float)(kLsVec + 1) / L.rf;
    g.s_scale = 1.0f / (L.rf * L.rf);
    return g;
}

template <typename T>
int ls_alloc(T **p, size_t count) {
    if (cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) {
        *p = nullptr;
        return MDG_ERR_CUDA;
    }
    return cudaMemset(*p, 0, sizeof(T) * std::max<size_t>(count, 1)) == cudaSuccess ? MDG_OK
                                                                                     : MDG_ERR_CUDA;
}

template <typename T>
void ls_dfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

}  // namespace

// Cells of edge >= rf + skin (at least 3 per axis), buffers for n atoms.
int ls_configure(mdg_system *s, float rf, float skin, int cap) {
    if (s->n_sys != 1) return MDG_ERR_INVALID;
    const SysDev &d = s->sys_h[0];
    int nc[3];
    for (int k = 0; k < 3; ++k) {
        nc[k] = (int)floor(d.Ld[k] / (double)(rf + skin));
        if (nc[k] < 3) return MDG_ERR_INVALID;
    }
    const bool keep = s->ls != nullptr;
    std::vector<float> old;
    Learned *L = s->ls;
    if (keep) {
        old.resize(kLsParams);
        cudaMemcpy(old.data(), L->params, sizeof(float) * kLsParams, cudaMemcpyDeviceToHost);
        ls_free(s);
    }
    L = new Learned();
    s->ls = L;
    L->configured = 1;
    L->rf = rf;
    L->skin = skin;
    L->cap = cap;
    for (int k = 0; k < 3; ++k) L->nc[k] = nc[k];
    L->n_cells = nc[0] * nc[1] * nc[2];
    L->n_tiles = (s->n + kLsTile - 1) / kLsTile;
    L->n_rows = L->n_tiles * kLsTile;
    const size_t n = s->n, rows = L->n_rows;
    int sms = s->n_sms > 0 ? s->n_sms : 1;
    L->n_gpart = std::min(2 * L->n_tiles, sms);
    L->n_red = (int)std::max<size_t>((rows + 255) / 256, 1);
    int rc = MDG_OK;
#define LA(ptr, cnt) \
    if (!rc) rc = ls_alloc(&(ptr), (cnt));
    LA(L->cell_of, n);
    LA(L->cell_count, L->n_cells);
    LA(L->cell_start, L->n_cells + 1);
    LA(L->cell_cursor, L->n_cells);
    LA(L->cell_atoms, n);
    LA(L->nlist, n);
    LA(L->list, (size_t)cap * n);
    LA(L->pos, n);
    LA(L->cpos, n);
    LA(L->xref, n);
    LA(L->slot_of, n);
    LA(L->flag, 2);
    for (int q = 0; q < 2; ++q) {
        LA(L->xraw[q], n * kLsFeat);
        LA(L->xb[q], rows * kLsFeat);
        LA(L->S[q], rows * 3 * kLsVec);
        LA(L->G[q], rows * 3);
        LA(L->Z1[q], rows * kLsHidden);
        LA(L->Z2[q], rows * kLsHidden);
        LA(L->T[q], n * 3);
    }
    LA(L->params, kLsParams);
    LA(L->wb, 2 * kLsWb);
    LA(L->adam_m, kLsParams);
    LA(L->adam_v, kLsParams);
    LA(L->dout, 2 * rows * kLsVec);
    LA(L->gpart, (size_t)L->n_gpart * kLsParams);
    LA(L->red, 2 * (size_t)L->n_red);
    LA(L->base, 3 * n);
    LA(L->J, 6 * n);
    LA(L->Jn, 6 * n);
    LA(L->x0, n);
    LA(L->fpos[0], n);
    LA(L->fpos[1], n);
    LA(L->fs, 3 * (size_t)s->n_pad);
    LA(L->mode, 2);
    LA(L->stats, 8);
    LA(L->done, 1);
#undef LA
    if (rc) {
        ls_free(s);
        return rc;
    }
    // identity normalisation, zero weights, unit output scale until set
    std::vector<float> p(kLsParams, 0.f);
    if (keep) p = old;
    else {
        for (int k = 0; k < kLsFeat; ++k) p[kLsSig + k] = 1.f;
        p[kLsScale] = 1.f;
    }
    if (cudaMemcpy(L->params, p.data(), sizeof(float) * kLsParams, cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return MDG_ERR_CUDA;
    if (cudaFuncSetAttribute(k_ls_mlp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kMlpSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_ls_mlp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kMlpSmem) != cudaSuccess ||
        cudaFuncSetAttribute(k_ls_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kBwdSmem) != cudaSuccess)
        return MDG_ERR_CUDA;
    rc = ls_tc_prepare(s);
    if (rc) return rc;
    if (ls_refresh_weights(s) != cudaSuccess) return MDG_ERR_CUDA;
    return cudaDeviceSynchronize() == cudaSuccess ? MDG_OK : MDG_ERR_CUDA;
}

void ls_free(mdg_system *s) {
    Learned *L = s->ls;
    if (!L) return;
    ls_dfree(L->cell_of);
    ls_dfree(L->cell_count);
    ls_dfree(L->cell_start);
    ls_dfree(L->cell_cursor);
    ls_dfree(L->cell_atoms);
    ls_dfree(L->nlist);
    ls_dfree(L->list);
    ls_dfree(L->pos);
    ls_dfree(L->cpos);
    ls_dfree(L->xref);
    ls_dfree(L->slot_of);
    ls_dfree(L->flag);
    for (int q = 0; q < 2; ++q) {
        ls_dfree(L->xraw[q]);
        ls_dfree(L->xb[q]);
        ls_dfree(L->S[q]);
        ls_dfree(L->G[q]);
        ls_dfree(L->Z1[q]);
        ls_dfree(L->Z2[q]);
        ls_dfree(L->T[q]);
    }
    ls_dfree(L->params);
    ls_dfree(L->wb);
    ls_dfree(L->adam_m);
    ls_dfree(L->adam_v);
    ls_dfree(L->dout);
    ls_dfree(L->gpart);
    ls_dfree(L->red);
    ls_dfree(L->base);
    ls_dfree(L->J);
    ls_dfree(L->Jn);
    ls_dfree(L->x0);
    ls_dfree(L->fpos[0]);
    ls_dfree(L->fpos[1]);
    ls_dfree(L->fs);
    ls_dfree(L->mode);
    ls_dfree(L->stats);
    ls_dfree(L->done);
    delete L;
    s->ls = nullptr;
}

cudaError_t ls_refresh_weights(mdg_system *s) {
    Learned &L = *s->ls;
    k_ls_wb<<<(kLsWb + 255) / 256, 256, 0, s->stream>>>(L);
    s->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return ls_mlp_tc(s, -1);  // -1: lay out the tensor-core operand copy
}

// Side-stream part of an evaluation (after PME): positions, the neighbour
// list at full evaluations, features, MLP.  Inner steps add base + G to f.
cudaError_t ls_side(mdg_system *s, int phase) {
    Learned &L = *s->ls;
    const Geo g = make_geo(s);
    const int n = s->n, tb = 256, nb = (n + tb - 1) / tb;
    const int slot = phase == kLsFrame ? s->ls_slot : 0;
    cudaStream_t st = s->stream;
    k_ls_pos<<<nb, tb, 0, st>>>(s->x, s->charge, L, g);
    // the list is rebuilt at the first step on which an atom has moved more
    // than half the skin since the last build (so no pair within rf is ever
    // missing), and always for an anchor or a training frame; otherwise the
    // build kernels return at once (they run beside the pair kernel)
    const int force = phase == kLsAnchor || phase == kLsFrame ? 1 : 0;
    k_ls_gate<<<1, 1, 0, st>>>(L, force);
    k_ls_cells<<<nb, tb, 0, st>>>(L, g);
    k_ls_scan<<<1, 1024, 0, st>>>(L);
    k_ls_scatter<<<nb, tb, 0, st>>>(L, n);
    k_ls_cellsort<<<(L.n_cells * 32 + 255) / 256, 256, 0, st>>>(L);
    k_ls_list<<<(n + 127) / 128, 128, 0, st>>>(L, g, s->partners, s->pw, s->status);
    s->launches += 7;
    const bool full = phase != kLsInner;
    const bool taylor = L.use_taylor && s->pme.order == 4 && g.phi;
    if (full && taylor) {  // the field-gradient term at this full evaluation
        k_ls_hessian<<<nb, tb, 0, st>>>(L, g);
        s->launches += 1;
        if (s->n_excl > 0) {
            k_ls_hessian_excl<<<(s->n_excl + 255) / 256, 256, 0, st>>>(L, g, s->excl_pairs,
                                                                       s->n_excl);
            s->launches += 1;
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const bool net = L.use_net || phase == kLsFrame;
    if (net) {
        const int gated = phase == kLsInner ? 1 : 0;
        const int fb = (n + kFeatThreads - 1) / kFeatThreads;
        if (phase == kLsFrame) k_ls_features<true><<<fb, kFeatThreads, 0, st>>>(L, g, slot, 0);
        else k_ls_features<false><<<fb, kFeatThreads, 0, st>>>(L, g, slot, gated);
        s->launches += 1;
        if (phase == kLsFrame) {
            k_ls_mlp<true><<<L.n_tiles, 256, kMlpSmem, st>>>(L, g, slot);
            s->launches += 1;
        } else if (L.use_tc) {
            e = ls_mlp_tc(s, 0);
        } else {
            k_ls_mlp<false><<<L.n_tiles, 256, kMlpSmem, st>>>(L, g, 0);
            s->launches += 1;
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (phase == kLsInner) {  // the predicted slow force joins the other forces
        k_ls_apply<<<nb, tb, 0, st>>>(L, g, s->inv_perm, s->f, taylor ? 1 : 0, L.use_net);
        s->launches += 1;
    }
    return cudaGetLastError();
}

// Main-stream part after the join: judge + combine at full evaluations of
// the learned form; the target copy of a training frame.
cudaError_t ls_after_join(mdg_system *s, int phase) {
    Learned &L = *s->ls;
    const Geo g = make_geo(s);
    const int tb = 256, nb = (s->n + tb - 1) / tb;
    if (phase == kLsFrame) {
        k_ls_target<<<nb, tb, 0, s->stream>>>(L, g, s->inv_perm, s->ls_slot);
        s->launches += 1;
        return cudaGetLastError();
    }
    if (phase != kLsOuter && phase != kLsAnchor) return cudaSuccess;
    const int taylor = L.use_taylor && s->pme.order == 4 && g.phi ? 1 : 0;
    k_ls_judge<<<nb, tb, 0, s->stream>>>(L, g, s->inv_perm, s->f, phase == kLsAnchor ? 1 : 0,
                                         L.done, taylor, L.use_net);
    k_ls_combine<<<nb, tb, 0, s->stream>>>(L, g, s->inv_perm, s->f, s->ls->k, L.use_net);
    s->launches += 2;
    return cudaGetLastError();
}

// Inference pass (no force update) on the features of `slot`, with the
// kernel the launch setting selects; G[slot] then holds the prediction.
cudaError_t ls_predict(mdg_system *s, int slot) {
    Learned &L = *s->ls;
    if (L.use_tc) return ls_mlp_tc(s, slot);
    const Geo g = make_geo(s);
    k_ls_mlp<false><<<L.n_tiles, 256, kMlpSmem, s->stream>>>(L, g, slot);
    s->launches += 1;
    return cudaGetLastError();
}

// One training step over the two recorded frames: loss, backward, Adam.
cudaError_t ls_train(mdg_system *s, float lr, int t, double *loss) {
    Learned &L = *s->ls;
    const Geo g = make_geo(s);
    cudaStream_t st = s->stream;
    const int nb = (s->n + 255) / 256;
    k_ls_residual<<<nb, 256, 0, st>>>(L, g);
    k_ls_dout<<<(L.n_rows + 255) / 256, 256, 0, st>>>(L, g, nb);
    cudaMemsetAsync(L.gpart, 0, sizeof(float) * (size_t)L.n_gpart * kLsParams, st);
    k_ls_backward<<<L.n_gpart, 256, kBwdSmem, st>>>(L, g);
    const float b1 = 0.9f, b2 = 0.999f;
    const double c1 = 1.0 - pow((double)b1, t), c2 = 1.0 - pow((double)b2, t);
    const float lr_t = (float)(lr * sqrt(c2) / c1);
    k_ls_adam<<<(kLsParams + 255) / 256, 256, 0, st>>>(L, L.n_gpart, lr_t, b1, b2, 1e-8f);
    s->launches += 4;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = ls_refresh_weights(s);
    if (e != cudaSuccess) return e;
    if (loss) {
        double v = 0.0;
        e = cudaMemcpyAsync(&v, L.stats + 5, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        *loss = v;
    }
    return e;
}

}  // namespace mdg
