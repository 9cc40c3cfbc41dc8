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

struct Pme {
    int on;
    int K[3];
    int order;
    double beta;
    long long *grid_i;  // K0*K1*K2 fixed point charge grid
    float *grid_r;      // real grid (FFT input, then potential)
    float2 *grid_c;     // K0*K1*(K2/2+1)
    float *influence;   // K0*K1*(K2/2+1)
    cufftHandle plan_f, plan_b;
    double e_self, e_net;  // FP64 constants of the Ewald sum
};

struct Graph {
    cudaGraphExec_t exec = nullptr;
    int steps = 0;
    unsigned mask = 0;
};

}  // namespace mdg

struct mdg_system {
    int device = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    int n = 0, n_pad = 0, n_clusters = 0;
    double box[3] = {0, 0, 0};

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
    long long *energy = nullptr;       // kEnergySlots
    int *status = nullptr;
    unsigned long long *stats = nullptr;  // 4 counters
    unsigned long long *step_dev = nullptr;
    double *fout = nullptr;            // (n,3) FP64 staging for get_forces

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
    mdg::Graph graph_step[2];          // one step: [0] plain, [1] starting with a re-sort
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
cudaError_t launch_nonbonded(mdg_system *s, unsigned mask, int energy, int dump);
cudaError_t launch_special(mdg_system *s, unsigned mask, int energy, int dump);
cudaError_t launch_pme(mdg_system *s, int energy, int *cufft_status);
cudaError_t launch_bonded(mdg_system *s, unsigned mask, int energy);
cudaError_t launch_integrate_pre(mdg_system *s);
cudaError_t launch_integrate_post(mdg_system *s, int energy);
cudaError_t launch_kinetic(mdg_system *s);
cudaError_t launch_forces_out(mdg_system *s);
cudaError_t launch_positions_out(mdg_system *s, double *out);
cudaError_t launch_noise(mdg_system *s, uint64_t step, float *out);
int prepare_sort_grid(mdg_system *s);   // host: column grid + cluster-order buffers
int pme_setup(mdg_system *s);           // host: grids, plans, influence function
void pme_free(mdg_system *s);
}  // namespace mdg
