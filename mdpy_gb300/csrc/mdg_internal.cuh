// mdg_internal.cuh -- shared definitions of libmdg's translation units.
//
// Data layout in HBM (per system; n atoms, cluster order holds n_pad slots =
// 32 * (ceil(n/32) + number of sort columns): every column is padded to whole
// clusters, so padding slots sit between columns):
//   x, v            double[n][3]        atom order (FP64 state, as mdpy's State)
//   f               int64 [3][n_pad]    cluster (sorted) order, fixed point 2^-32,
//                                       SoA so a cluster's 32 atoms are one
//                                       coalesced 256-byte segment per axis
//   xq              float4[n_pad]       sorted order: x, y, z, q*sqrt(k_e);
//                                       padding slots sit at 1e18 A with q = 0
//   prm             float2[n_pad]       sorted order: sigma/2, sqrt(4 eps)
//   bbox            float4[2][clusters] centre (w = #atoms) and half extents
//   partners        int[n_pad][pw]      sorted order: 1-2/1-3/1-4 partners of
//                                       each atom (sorted indices, -1 padded)
//   energy          int64[16]           fixed point 2^-32 per term + kinetic
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <vector>

#include "../../include/mdg.h"

namespace mdg {

constexpr int kCluster = 32;
constexpr double kFixScale = 4294967296.0;  // 2^32
constexpr float kFixScaleF = 4294967296.0f;
constexpr double kFixInv = 1.0 / 4294967296.0;
constexpr float kFarAway = 1.0e18f;
constexpr float kFixLimit = 1.0e9f;  // |contribution| above this overflows int64 sums
constexpr int kEnergySlots = 16;
constexpr int kSlotKinetic = 8;
constexpr int kStatus = 0;

// status bits raised by kernels (bit = MDG_ERR_* code)
__device__ __forceinline__ void raise_status(int *status, int code) {
    atomicOr(status, 1 << code);
}

__device__ __forceinline__ long long to_fix(float v) { return __float2ll_rn(v * kFixScaleF); }
__device__ __forceinline__ long long to_fix_d(double v) { return __double2ll_rn(v * kFixScale); }

// fire-and-forget 64-bit add into a fixed-point accumulator (two's complement)
__device__ __forceinline__ void fix_red(unsigned long long *p, long long v) {
    atomicAdd(p, (unsigned long long)v);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adds this thread's FP64 energy terms v[t] to energy[sys * kEnergySlots +
// slot[t]] (sys < 0: nothing to add).  Every thread of the block must call it
// (it holds a block barrier); blockDim.x is a multiple of 32.  When all
// contributing threads belong to one system -- always, for a single system --
// the block sums in FP64 and issues one atomic per term; a block that spans
// systems issues one atomic per term and warp (one per lane for a warp that
// itself spans systems).  The fixed-point sums stay order independent.
template <int NT>
__device__ void block_energy_add(long long *energy, int sys, const double (&v)[NT],
                                 const int (&slot)[NT]) {
    __shared__ double s_e[NT][32];
    __shared__ int s_sys[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned act = __ballot_sync(0xffffffffu, sys >= 0);
    int wsys = act ? __shfl_sync(0xffffffffu, sys, __ffs(act) - 1) : -1;
    const bool uni = __all_sync(0xffffffffu, sys < 0 || sys == wsys);
    double r[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) r[t] = warp_sum_d(sys >= 0 ? v[t] : 0.0);
    if (!uni) {
#pragma unroll
        for (int t = 0; t < NT; ++t)
            if (sys >= 0 && v[t] != 0.0)
                fix_red((unsigned long long *)&energy[sys * kEnergySlots + slot[t]],
                        to_fix_d(v[t]));
        wsys = -1;  // added lane by lane
    }
    if (lane == 0) {
        s_sys[w] = wsys;
#pragma unroll
        for (int t = 0; t < NT; ++t) s_e[t][w] = r[t];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int bsys = -1;
        bool buni = true;
        for (int k = 0; k < nw; ++k) {
            const int q = s_sys[k];
            if (q < 0) continue;
            if (bsys < 0) bsys = q;
            else if (q != bsys) buni = false;
        }
        if (bsys >= 0 && buni) {
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                double a = 0.0;
                for (int k = 0; k < nw; ++k)
                    if (s_sys[k] >= 0) a += s_e[t][k];
                if (a != 0.0)
                    fix_red((unsigned long long *)&energy[bsys * kEnergySlots + slot[t]],
                            to_fix_d(a));
            }
        } else if (!buni) {
            for (int k = 0; k < nw; ++k) {
                const int q = s_sys[k];
                if (q < 0) continue;
#pragma unroll
                for (int t = 0; t < NT; ++t)
                    if (s_e[t][k] != 0.0)
                        fix_red((unsigned long long *)&energy[q * kEnergySlots + slot[t]],
                                to_fix_d(s_e[t][k]));
            }
        }
    }
}

struct SysDev;

// Per-step packing of one 32-slot cluster into the float copy the force
// kernels read (see pack_cluster below).
struct PackArgs {
    const double *x;
    const int *perm;
    const float *q_sorted;
    int n_clusters, n_pad;
    float4 *xq;
    float4 *bbox;
    float4 *hbox;   // boxes of the two 16-slot halves: centre, half extents (x2)
    float4 *qbox;   // boxes of the four 8-slot quarters: centre, half extents (x4)
    unsigned long long *f;
    const SysDev *sys;
    const int *cl_sys, *cl_col, *col_xy;
    float *overhang;
};

// per-system parameters, read by kernels through a device table (one entry
// per independent system of a batch; a single system is a batch of one)
struct SysDev {
    float L[3], invL[3];    // box edges (A) and inverses
    double Ld[3];           // FP64 box for the FP64 minimum image
    double invLd[3];        // and its inverse (GB300's FP64 divide is slow)
    int atom_off, n_atoms;  // atom range
    int cl_off, cl_cap;     // cluster range (capacity: ceil(n/32) + columns)
    int col_off, n_cols;    // sort columns
    int key_off, nzb;       // sort keys: (column, height bin)
    int ncx, ncy;           // column grid
    int col_mode;           // pair search over neighbouring columns (else all clusters)
    int K[3];               // PME grid
    float kl[3];            // K / L
    long long grid_off;     // offset of this system's real PME grid (elements)
    long long cgrid_off;    // offset of its complex grid and influence function
};

// Pair-set parity mode (the pair dump only): the reference's own pair test
// in its float32 arithmetic.  The FP64 state is first put in the reference's
// frame by mdpy's wrap (x - L round(x / L) with the float32 inverse box,
// mdpy/utils/pbc.py:28-36 -- the positions mdg_get_positions reports) and
// rounded to float32 (mdpy's positions are float32); then d
// = x_j - x_i, scaled by the float32 inverse box, minus its rounded value,
// scaled back (unwrap_vec, pbc.py:38-43), and r = sqrt of the left-to-right
// sum of squares (np.linalg.norm, charmm_nonbonded_constraint.py:85-90),
// every operation rounded once (no fused multiply-add), compared with rc.
__device__ __forceinline__ bool ref_within32(const double *x, int i, int j, const SysDev &sd,
                                             float rc) {
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double Ld = sd.Ld[k];
        const double inv32 = (double)(float)(1.0 / Ld);
        const double xi = x[3 * i + k] - Ld * rint(x[3 * i + k] * inv32);
        const double xj = x[3 * j + k] - Ld * rint(x[3 * j + k] * inv32);
        const float L = (float)Ld;
        float sc = __fmul_rn(__fsub_rn((float)xj, (float)xi), __frcp_rn(L));
        sc = __fsub_rn(sc, rintf(sc));
        d[k] = __fmul_rn(sc, L);
    }
    const float r2 =
        __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
    return __fsqrt_rn(r2) <= rc;
}

// systems sharing one PME grid size: one batched cuFFT plan pair
struct PmeGroup {
    int K[3];
    int count;
    long long grid_off, cgrid_off;
    long long nr_stride, nc_stride;  // elements between members' grids (padded)
    cufftHandle plan_f = 0, plan_b = 0;
    int *sys_ids = nullptr;  // device: the group's system ids, in grid order
};

struct Pme {
    int on = 0;
    int order = 4;
    double beta = 0.0;
    long long grid_total = 0, cgrid_total = 0;
    long long *grid_i = nullptr;  // fixed-point charge grids, all systems
    float *grid_r = nullptr;      // real grids (FFT input, then potential)
    float2 *grid_c = nullptr;     // half-spectrum complex grids
    float *influence = nullptr;   // influence functions, complex-grid layout
    std::vector<PmeGroup> groups;
};

// One warp packs cluster `warp`; lane slot k holds atom position c (FP64)
// when valid.  Writes the float copy (x, y, z, q sqrt(k_e)), zeroes the
// slot's force words, and lane 0 writes the cluster box and raises the
// system's overhang (how far boxes reach out of their sort columns).
// Between re-sorts the FP64 positions drift freely out of [0, L).  The pair
// search tries the images -1, 0, +1 of each cluster pair, which is exact
// while every stored coordinate stays within a window of width 1.5 L: a
// coordinate that leaves [-L/4, 5L/4) is wrapped back into [0, L) here (its
// cluster box then spans the box, and the search covers it with all 27
// images).
__device__ __forceinline__ void pack_cluster(const PackArgs &a, int warp, int k, bool valid,
                                             double (&c)[3]) {
    const int lane = threadIdx.x & 31;
    float4 p;
    if (valid) {
        const double *Ld = a.sys[a.cl_sys[warp]].Ld;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (c[d] < -0.25 * Ld[d] || c[d] >= 1.25 * Ld[d]) c[d] -= Ld[d] * floor(c[d] / Ld[d]);
        p = make_float4((float)c[0], (float)c[1], (float)c[2], a.q_sorted[k]);
    } else {
        p = make_float4(kFarAway, kFarAway, kFarAway, 0.0f);
    }
    a.xq[k] = p;
    a.f[k] = 0ull;
    a.f[a.n_pad + k] = 0ull;
    a.f[2 * a.n_pad + k] = 0ull;
    float lox = valid ? p.x : INFINITY, loy = valid ? p.y : INFINITY, loz = valid ? p.z : INFINITY;
    float hix = valid ? p.x : -INFINITY, hiy = valid ? p.y : -INFINITY,
          hiz = valid ? p.z : -INFINITY;
    const unsigned vb = __ballot_sync(0xffffffffu, valid);
    // the four 8-slot quarters first, then the two 16-slot halves, then the
    // whole cluster
#pragma unroll
    for (int o = 1; o <= 16; o <<= 1) {
        lox = fminf(lox, __shfl_xor_sync(0xffffffffu, lox, o));
        loy = fminf(loy, __shfl_xor_sync(0xffffffffu, loy, o));
        loz = fminf(loz, __shfl_xor_sync(0xffffffffu, loz, o));
        hix = fmaxf(hix, __shfl_xor_sync(0xffffffffu, hix, o));
        hiy = fmaxf(hiy, __shfl_xor_sync(0xffffffffu, hiy, o));
        hiz = fmaxf(hiz, __shfl_xor_sync(0xffffffffu, hiz, o));
        if (o == 4 && (lane & 7) == 0) {
            const int qg = lane >> 3;
            const bool any = (vb >> (8 * qg)) & 0xffu;
            a.qbox[8 * warp + 2 * qg] =
                any ? make_float4(0.5f * (lox + hix), 0.5f * (loy + hiy), 0.5f * (loz + hiz), 1.0f)
                    : make_float4(kFarAway, kFarAway, kFarAway, 0.0f);
            a.qbox[8 * warp + 2 * qg + 1] =
                any ? make_float4(0.5f * (hix - lox), 0.5f * (hiy - loy), 0.5f * (hiz - loz), 0.0f)
                    : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        if (o == 8 && (lane & 15) == 0) {
            const int h = lane >> 4;
            const bool any = (vb >> (16 * h)) & 0xffffu;
            a.hbox[4 * warp + 2 * h] =
                any ? make_float4(0.5f * (lox + hix), 0.5f * (loy + hiy), 0.5f * (loz + hiz), 1.0f)
                    : make_float4(kFarAway, kFarAway, kFarAway, 0.0f);
            a.hbox[4 * warp + 2 * h + 1] =
                any ? make_float4(0.5f * (hix - lox), 0.5f * (hiy - loy), 0.5f * (hiz - loz), 0.0f)
                    : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
    const int cnt = __popc(vb);
    if (lane == 0) {
        if (cnt == 0) {  // an all-padding cluster: far away, zero extent
            a.bbox[2 * warp] = make_float4(kFarAway, kFarAway, kFarAway, 0.0f);
            a.bbox[2 * warp + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            a.bbox[2 * warp] = make_float4(0.5f * (lox + hix), 0.5f * (loy + hiy),
                                           0.5f * (loz + hiz), (float)cnt);
            a.bbox[2 * warp + 1] = make_float4(0.5f * (hix - lox), 0.5f * (hiy - loy),
                                               0.5f * (hiz - loz), 0.0f);
            const int col = a.cl_col[warp];
            if (col >= 0) {
                const int q = a.cl_sys[warp];
                const SysDev &d = a.sys[q];
                const int pk = a.col_xy[col];
                const float ax = d.L[0] / (float)d.ncx, ay = d.L[1] / (float)d.ncy;
                const float x0 = (float)(pk >> 16) * ax, y0 = (float)(pk & 0xffff) * ay;
                const float ov = fmaxf(fmaxf(fmaxf(x0 - lox, hix - (x0 + ax)),
                                             fmaxf(y0 - loy, hiy - (y0 + ay))),
                                       0.0f);
                if (ov > a.overhang[q])
                    atomicMax((unsigned int *)&a.overhang[q], __float_as_uint(ov));
            }
        }
    }
}

struct Graph {
    cudaGraphExec_t exec = nullptr;
    int steps = 0;
    unsigned mask = 0;
};

// ---- learned slow force (multiple time steps) ------------------------------
// Per atom i: 64 invariant features (32 cubic B-spline radial bins, channels
// sum_j q_j phi_b(r_ij) and sum_j phi_b(r_ij), j within rf), a BF16 MLP
// 64 -> 128 -> 128 -> 16 (SiLU, FP32 accumulation) giving coefficients C_ib
// on 16 vector basis functions S_ib = q_i sum_j q_j psi_b(r_ij) d_ij / rf^2,
// and the predicted slow force G_i = sum_b C_ib S_ib (rotation equivariant).
constexpr int kLsBins = 32;
constexpr int kLsFeat = 2 * kLsBins;
constexpr int kLsVec = 16;
constexpr int kLsHidden = 128;
constexpr int kLsTile = 128;  // atoms per MLP tile
// the parameter vector (FP32): feature shift and inverse scale, the three
// layers (weights stored [in][out]), the output scale
constexpr int kLsMu = 0;
constexpr int kLsSig = kLsMu + kLsFeat;
constexpr int kLsW1 = kLsSig + kLsFeat;
constexpr int kLsB1 = kLsW1 + kLsFeat * kLsHidden;
constexpr int kLsW2 = kLsB1 + kLsHidden;
constexpr int kLsB2 = kLsW2 + kLsHidden * kLsHidden;
constexpr int kLsW3 = kLsB2 + kLsHidden;
constexpr int kLsB3 = kLsW3 + kLsHidden * kLsVec;
constexpr int kLsScale = kLsB3 + kLsVec;
constexpr int kLsParams = kLsScale + 1;
// BF16 weight copies: W1, W2, W3 in [in][out] order, then the same three in
// the tensor-core operand layout (see mdg_learned_tc.cu)
constexpr int kLsWb = kLsFeat * kLsHidden + kLsHidden * kLsHidden + kLsHidden * kLsVec;

// element (r, k) of a K-major BF16 operand with R rows (R, K multiples of
// 8), as the tensor cores read it from shared memory without swizzle: 8 x 8
// core matrices of 128 contiguous bytes, K-chunk-major
__host__ __device__ constexpr int ls_tc_off(int r, int k, int R) {
    return ((k >> 3) * (R >> 3) + (r >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}
// features of atom row i inside the tile-major feature array
__host__ __device__ constexpr size_t ls_xoff(int i, int k) {
    return (size_t)(i / kLsTile) * kLsTile * kLsFeat + ls_tc_off(i % kLsTile, k, kLsTile);
}

enum LsPhase { kLsOff = 0, kLsInner = 1, kLsOuter = 2, kLsAnchor = 3, kLsFrame = 4 };
enum LsMode { kLsLearned = 0, kLsImpulse = 1 };

struct Learned {
    int configured = 0, enabled = 0, trained = 0;
    int k = 4;                 // outer step
    float threshold = 1e-3f;   // judge: relative force error that switches to the fallback
    float rf = 6.0f, skin = 1.0f;
    int cap = 256;             // neighbour list entries per atom
    int nc[3] = {0, 0, 0}, n_cells = 0;
    int n_rows = 0, n_tiles = 0;  // MLP rows (atoms padded to whole tiles)
    int use_tc = 1;            // tensor-core (tcgen05) inference kernel (0: SIMT)
    int use_taylor = 0;        // field-gradient term J (x - x0) in the prediction
    int use_net = 1;           // the network's G(x) - G(x0) in the prediction
    int tc_wait_test = 0;      // one-shot test of the tcgen05 kernel's bounded waits (see
                               // mdg_learned_wait_test)
    int *cell_of = nullptr, *cell_count = nullptr, *cell_start = nullptr,
        *cell_cursor = nullptr, *cell_atoms = nullptr;
    int *nlist = nullptr, *list = nullptr;  // per slot of the cell order; list: [cap][n]
    float4 *pos = nullptr;     // wrapped FP32 positions, q sqrt(k_e) (atom order)
    float4 *cpos = nullptr;    // the same in cell order (list build)
    float4 *xref = nullptr;    // positions at the last list build (motion test)
    int *slot_of = nullptr;    // atom -> its slot in the cell order of the last build
    int *flag = nullptr;       // [0]: rebuild requested, [1]: rebuilding now
    float *xraw[2] = {nullptr, nullptr};  // raw features of training frames (n x 64)
    uint16_t *xb[2] = {nullptr, nullptr};  // normalised BF16 features, tiles (ls_xoff)
    float *S[2] = {nullptr, nullptr};      // vector basis [rows][48] (3 b + axis)
    float *G[2] = {nullptr, nullptr};      // predicted slow force [3][rows]
    float *Z1[2] = {nullptr, nullptr}, *Z2[2] = {nullptr, nullptr};  // training
    float *T[2] = {nullptr, nullptr};      // slow-force targets [3][n]
    float *params = nullptr;   // FP32 master
    uint16_t *wb = nullptr;    // BF16 copies (2 * kLsWb)
    float *adam_m = nullptr, *adam_v = nullptr, *grad = nullptr;
    float *dout = nullptr;     // [2][rows][16] training gradients at the outputs
    float *gpart = nullptr;    // per-CTA gradient partials
    int n_gpart = 0;
    double *red = nullptr;     // reduction partials
    int n_red = 0;
    long long *base = nullptr; // F_slow(t0) - G(t0), fixed point [3][n]
    long long *J = nullptr;    // d F_slow / d x_i at t0 (xx, yy, zz, xy, xz, yz), fixed [6][n]
    long long *Jn = nullptr;   // the same at the current full evaluation
    float4 *x0 = nullptr;      // positions at t0
    float4 *fpos[2] = {nullptr, nullptr};  // positions of the training frames
    unsigned long long *fs = nullptr;  // slow force of an outer step (sorted, fixed point)
    int *mode = nullptr;       // LsMode of the current interval
    double *stats = nullptr;   // last error, max error, sum of errors, judged, fallbacks,
                               // last loss, last target norm
    int *done = nullptr;       // block counter of the judge's last-block reduction
};

}  // namespace mdg

struct mdg_system {
    int device = 0;
    int n_sys = 1;                     // independent systems in this batch
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // side stream for the work that runs beside the pair kernel (PME, special
    // pairs, bonded terms), joined back through two events
    // PME runs on side_stream, special pairs and bonded terms on bond_stream,
    // both beside the pair kernel; each pair of streams: normal, highest priority
    cudaStream_t side_stream = nullptr, bond_stream = nullptr;
    cudaStream_t side_streams[2] = {nullptr, nullptr}, bond_streams[2] = {nullptr, nullptr};
    cudaEvent_t ev_join2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int n = 0, n_pad = 0, n_clusters = 0;
    std::vector<mdg::SysDev> sys_h;    // host copy of the system table
    mdg::SysDev *sys_dev = nullptr;    // device system table
    std::vector<int> atoms_per_sys;
    std::vector<double> e_self, e_net; // FP64 Ewald constants per system
    std::vector<double> qsum, q2sum;   // per-system charge sums (e)
    int *atom_sys = nullptr;           // per atom: system id
    int *cl_sys = nullptr;             // per cluster slot: system id
    int *col_sys = nullptr;            // per sort column: system id
    int *cl_col = nullptr;             // per cluster slot: global sort column (-1: none)
    int *col_xy = nullptr;             // per global sort column: (cx << 16) | cy
    float *overhang = nullptr;         // per system: how far (A) cluster boxes reach out
                                       // of their columns since the last re-sort

    // static, atom order
    double *mass = nullptr, *inv_mass = nullptr;
    float *charge = nullptr;          // q * sqrt(k_e)
    float4 *lj = nullptr;             // sigma/2, sqrt(4 eps), sigma14/2, sqrt(4 eps14)
    int pw = 0;                       // partner width
    int *partners = nullptr;          // atom order, (n, pw); bit 30 set for 1-4
    int n_excl = 0, n_14 = 0;
    int2 *excl_pairs = nullptr;       // unique i<j 1-2/1-3 pairs (atom order)
    int2 *pairs14 = nullptr;          // unique i<j 1-4 pairs
    int have_masses = 0, have_charges = 0, have_lj = 0, have_x = 0, have_v = 0;

    // cluster order (rebuilt by reorder)
    int *perm = nullptr, *inv_perm = nullptr;
    float *q_sorted = nullptr;
    float2 *prm_sorted = nullptr;
    int *partners_sorted = nullptr;
    int2 *cluster_partner_range = nullptr;

    // spatial sort scratch: ncell = (columns x, columns y, height bins);
    // n_cells = number of (column, height bin) keys
    int ncell[3] = {0, 0, 0};
    int n_cells = 0;
    int n_cols = 0;
    int *col_ncl = nullptr, *col_cl_start = nullptr;
    int *cell_rank = nullptr, *cell_count = nullptr, *cell_start = nullptr,
        *cell_cursor = nullptr, *atom_key = nullptr, *tmp_perm = nullptr, *scan_blocks = nullptr;
    int n_scan_blocks = 0;

    // per step
    double *x = nullptr, *v = nullptr;
    unsigned long long *f = nullptr;   // 3 * n_pad fixed point
    float4 *xq = nullptr;
    float4 *bbox = nullptr;
    float4 *hbox = nullptr;            // float4[4][clusters]: boxes of the 16-slot halves
    float4 *qbox = nullptr;            // float4[8][clusters]: boxes of the 8-slot quarters
    long long *energy = nullptr;       // kEnergySlots per system
    int *status = nullptr;
    unsigned long long *stats = nullptr;  // 4 counters
    unsigned long long *step_dev = nullptr;
    double *fout = nullptr;            // (n,3) FP64 staging for get_forces
    long long *host_stage = nullptr;   // pinned host staging of mdg_step_host
    double *xin = nullptr;             // mdg_step_host: incoming positions (3n)
    double *vsave = nullptr;           // and the velocities before a speculative step
    int *same_flag = nullptr;          // and their comparison with the state
    // energy snapshots (mdg_energy_snapshot): pinned ring of slots of
    // kEnergySlots * n_sys energy words + the status word, one event each
    long long *snap_host = nullptr;
    cudaEvent_t snap_ev[MDG_SNAPSHOT_SLOTS] = {};
    unsigned snap_mask[MDG_SNAPSHOT_SLOTS] = {};  // forces_mask at the snapshot
    bool snap_recip[MDG_SNAPSHOT_SLOTS] = {};     // PME energy in the words
    bool snap_taken[MDG_SNAPSHOT_SLOTS] = {};

    // launch shapes (set by hand or by mdg_autotune): work items per
    // i-cluster, persistent work-queue form, PME spread/gather block size
    int nb_split = 4;
    int nb_persistent = 0;            // 0: one CTA per item; else resident CTAs per SM
    int nb_persistent_ctas = 0;       // SMs x nb_persistent
    int n_sms = 0;
    int *nb_queue = nullptr;
    int pme_block = 256;
    int side_priority = 0;            // 1: side stream at the highest priority
    int nb_split_rings = 1;           // 1: charge-only j atoms sweep without LJ
    int pme_tiles = 0;                // bit 0: tiled spread, bit 1: tiled gather
    int nb_half = 0;                  // 1: 16-atom i groups per half warp

    // multiple time steps (impulse): the reciprocal-space force enters every
    // mts_k-th evaluation with weight mts_k and is skipped in between
    int mts_k = 1;
    float recip_weight = 1.0f;        // weight of the reciprocal force in the next evaluation
    float forces_weight = 1.0f;       // weight in the force buffer's evaluation
                                      // (-1: forces of the learned slow-force form)
    // learned slow force: what the next evaluation does for it (mdg::LsPhase),
    // and where PME and the excluded-pair correction put their forces (null: f)
    mdg::Learned *ls = nullptr;
    int ls_phase = 0;
    int ls_slot = 0;
    unsigned long long *slow_target = nullptr;

    // nonbonded configuration
    float cutoff = 12.0f, rswitch = 0.0f;
    int lj_on = 1, coul_mode = MDG_COUL_NONE;
    double beta = 0.0;
    int nb_configured = 0;

    mdg::Pme pme{};

    // bonded
    int nb = 0, na = 0, nd = 0, ni = 0;
    int2 *bond_idx = nullptr;
    float2 *bond_prm = nullptr;
    int4 *angle_idx = nullptr;
    float4 *angle_prm = nullptr;
    int4 *dih_idx = nullptr;
    float4 *dih_prm = nullptr;
    int4 *imp_idx = nullptr;
    float2 *imp_prm = nullptr;

    // integrator
    int integ_kind = -1;
    double dt = 1.0, temperature = 300.0, friction = 0.0;
    uint64_t seed = 0;
    uint64_t step = 0;

    // bookkeeping
    int need_reorder = 1;
    int reorder_interval = 20;
    int steps_since_reorder = 0;
    int forces_valid = 0;
    int evaluated_once = 0;
    unsigned forces_mask = 0;
    long long launches = 0;
    mdg::Graph graph;                  // chunk of reorder_interval steps
    mdg::Graph graph_step[2][2][2];    // one step: [re-sort first][with energies][MTS outer boundary]
    mdg::Graph graph_eval[2];          // the evaluation before a first step: [re-sort first]
    int graph_mode = 0;

    // pair dump
    int *dump_buf = nullptr;
    int64_t dump_cap = 0;
    unsigned long long *dump_count = nullptr;
};

// ---- launch helpers shared by the translation units -----------------------
namespace mdg {
// each returns cudaError_t of the launch
cudaError_t launch_reorder(mdg_system *s);
cudaError_t launch_pack(mdg_system *s);
PackArgs make_pack_args(mdg_system *s);
cudaError_t launch_nonbonded(mdg_system *s, unsigned mask, int energy, int dump);
cudaError_t launch_special(mdg_system *s, unsigned mask, int energy, int dump);
cudaError_t launch_pme(mdg_system *s, int energy, int *cufft_status);
cudaError_t launch_bonded(mdg_system *s, unsigned mask, int energy);
cudaError_t launch_integrate_pre(mdg_system *s);
cudaError_t launch_integrate_post(mdg_system *s, int energy);
cudaError_t launch_kinetic(mdg_system *s);
cudaError_t launch_forces_out(mdg_system *s);
cudaError_t launch_positions_out(mdg_system *s, double *out);
cudaError_t launch_same_positions(mdg_system *s, const double *xin, int *flag);
cudaError_t launch_noise(mdg_system *s, uint64_t step, float *out);
cudaError_t launch_sd_step(mdg_system *s, double alpha);
int prepare_sort_grid(mdg_system *s);   // host: column grid + cluster-order buffers
int pme_setup(mdg_system *s, const int *grids);  // host: grids, plans, influence functions
int upload_sys_table(mdg_system *s);
void pme_free(mdg_system *s);
cudaError_t noalloc_scratch(int device, long long **out);  // static scratch of the no-alloc path
cudaError_t launch_kinetic_scratch(mdg_system *s, long long *acc);
// learned slow force (mdg_learned.cu)
int ls_configure(mdg_system *s, float rf, float skin, int cap);
void ls_free(mdg_system *s);
cudaError_t ls_side(mdg_system *s, int phase);   // side stream: features, MLP, forces
cudaError_t ls_after_join(mdg_system *s, int phase);  // main stream: judge, combine, targets
cudaError_t ls_refresh_weights(mdg_system *s);
cudaError_t ls_train(mdg_system *s, float lr, int t, double *loss);
cudaError_t ls_predict(mdg_system *s, int slot);
cudaError_t ls_mlp_tc(mdg_system *s, int slot);  // mdg_learned_tc.cu
int ls_tc_prepare(mdg_system *s);
}  // namespace mdg
