// mdg_sort.cu -- spatial sort of atoms into 32-atom clusters, and the per-step
// pack of cluster coordinates and bounding boxes.
//
// Replaces mdpy's CellList (mdpy/core/cell_list.py:83-116), which rebuilds a
// dense padded (nx, ny, nz, max_per_cell) cell list from scratch on every
// State.set_positions.  Here the atoms are re-sorted every `reorder_interval`
// steps into columns: the box is cut into an x-y grid of columns whose cross
// section is the edge a = (32/rho)^(1/3) of a cube holding 32 atoms, atoms are
// ordered by height inside each column, and every column is padded to a whole
// number of 32-atom clusters.  A cluster is then a compact ~a x a x a block
// (a ~ 7 A in water), which keeps the pair kernel's bounding-box candidates
// tight.  Columns are visited in 2-D Z-order so that neighbouring clusters
// have nearby indices.  Between sorts only the bounding boxes are refreshed
// (k_pack); neighbour candidates are found from those boxes in the pair
// kernel, so the sort interval affects efficiency only, never which pairs
// are found.
//
// The sort is a deterministic counting sort over (column, height bin) keys:
// histogram, exclusive scan, scatter, then an insertion sort by atom index
// inside each (small) bin, so a given configuration always yields the same
// order.  Padding slots carry perm = -1, charge 0 and a far-away position.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mdg_internal.cuh"

namespace mdg {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanPerBlock = 2 * kScanThreads;

__global__ void k_bin(double *__restrict__ x, int n, const SysDev *__restrict__ sys,
                      const int *__restrict__ atom_sys, const int *__restrict__ col_rank,
                      int *__restrict__ key, int *__restrict__ count, int *__restrict__ status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SysDev &d = sys[atom_sys[i]];
    const int nc[3] = {d.ncx, d.ncy, d.nzb};
    int c[3];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double L = d.Ld[k];
        double p = x[3 * i + k];
        // particle loss as mdpy's wrap_positions defines it (mdpy/utils/pbc.py:
        // 30-34): a non-finite coordinate, or one two or more box lengths
        // from the central image (|round(x / L)| >= 2)
        ok = ok && isfinite(p) && fabs(rint(p * d.invLd[k])) < 2.0;
        p -= L * floor(p / L);
        if (p >= L) p -= L;
        if (!(p >= 0.0)) p = 0.0;
        x[3 * i + k] = p;
        int b = (int)(p * (nc[k] / L));
        c[k] = b < 0 ? 0 : (b >= nc[k] ? nc[k] - 1 : b);
    }
    if (!ok) raise_status(status, MDG_ERR_PARTICLE_LOSS);
    const int k = d.key_off + col_rank[d.col_off + c[0] * d.ncy + c[1]] * d.nzb + c[2];
    key[i] = k;
    atomicAdd(&count[k], 1);
}

// exclusive scan of two values per thread over a 1024-thread block
__device__ void block_scan2(int a, int b, int &ea, int &eb, int &total) {
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = a + b, inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        int t = warp_tot[lane], ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += u;
        }
        warp_tot[lane] = ti - t;  // exclusive
        __syncwarp();
    }
    __syncthreads();
    int base = warp_tot[w];
    int excl = base + inc - s;
    ea = excl;
    eb = excl + a;
    // block total: last thread's inclusive
    __shared__ int tot;
    if (threadIdx.x == blockDim.x - 1) tot = excl + s;
    __syncthreads();
    total = tot;
    __syncthreads();
}

__global__ void k_block_sums(const int *__restrict__ in, int n, int *__restrict__ sums) {
    int base = blockIdx.x * kScanPerBlock + 2 * threadIdx.x;
    int a = base < n ? in[base] : 0, b = base + 1 < n ? in[base + 1] : 0;
    int ea, eb, tot;
    block_scan2(a, b, ea, eb, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_top(int *sums, int nblocks) {
    int carry = 0;
    for (int off = 0; off < nblocks; off += kScanPerBlock) {
        int i = off + 2 * threadIdx.x;
        int a = i < nblocks ? sums[i] : 0, b = i + 1 < nblocks ? sums[i + 1] : 0;
        int ea, eb, tot;
        block_scan2(a, b, ea, eb, tot);
        if (i < nblocks) sums[i] = carry + ea;
        if (i + 1 < nblocks) sums[i + 1] = carry + eb;
        carry += tot;
        __syncthreads();
    }
}

__global__ void k_scan_final(const int *__restrict__ in, int n, const int *__restrict__ sums,
                             int *__restrict__ out) {
    int base = blockIdx.x * kScanPerBlock + 2 * threadIdx.x;
    int a = base < n ? in[base] : 0, b = base + 1 < n ? in[base + 1] : 0;
    int ea, eb, tot;
    block_scan2(a, b, ea, eb, tot);
    int off = sums[blockIdx.x];
    if (base < n) out[base] = off + ea;
    if (base + 1 < n) out[base + 1] = off + eb;
    // the element past the end receives the grand total
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = off + tot;
}

__global__ void k_scatter(const int *__restrict__ key, int n, const int *__restrict__ start,
                          int *__restrict__ cursor, int *__restrict__ tmp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = key[i];
    int slot = atomicAdd(&cursor[k], 1);
    tmp[start[k] + slot] = i;
}

// deterministic order inside each cell: ascending atom index
__global__ void k_cell_sort(const int *__restrict__ start, int ncells, int *__restrict__ tmp) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = start[c], e = start[c + 1];
    for (int i = b + 1; i < e; ++i) {
        int v = tmp[i], j = i - 1;
        while (j >= b && tmp[j] > v) {
            tmp[j + 1] = tmp[j];
            --j;
        }
        tmp[j + 1] = v;
    }
}

// clusters per column (columns of each system in rank order), then the
// exclusive scan over all columns of all systems
__global__ void k_col_clusters(const int *__restrict__ start, int n_cols,
                               const SysDev *__restrict__ sys, const int *__restrict__ col_sys,
                               int *__restrict__ col_ncl) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cols) return;
    const SysDev &d = sys[col_sys[c]];
    const int lc = c - d.col_off;
    const int cnt = start[d.key_off + (lc + 1) * d.nzb] - start[d.key_off + lc * d.nzb];
    col_ncl[c] = (cnt + kCluster - 1) / kCluster;
}

__global__ void k_col_scan(const int *__restrict__ col_ncl, int n_cols,
                           int *__restrict__ col_cl_start) {
    int carry = 0;
    for (int off = 0; off < n_cols; off += kScanPerBlock) {
        int i = off + 2 * threadIdx.x;
        int a = i < n_cols ? col_ncl[i] : 0, b = i + 1 < n_cols ? col_ncl[i + 1] : 0;
        int ea, eb, tot;
        block_scan2(a, b, ea, eb, tot);
        if (i < n_cols) col_cl_start[i] = carry + ea;
        if (i + 1 < n_cols) col_cl_start[i + 1] = carry + eb;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) col_cl_start[n_cols] = carry;
}

// every cluster of a column learns its column (clusters past a column's
// atoms, and past a system's used clusters, keep -1)
__global__ void k_cluster_columns(const int *__restrict__ col_ncl,
                                  const int *__restrict__ col_cl_start, int n_cols,
                                  const SysDev *__restrict__ sys, const int *__restrict__ col_sys,
                                  int *__restrict__ cl_col) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cols) return;
    const SysDev &d = sys[col_sys[c]];
    const int first = d.cl_off + col_cl_start[c] - col_cl_start[d.col_off];
    for (int k = 0; k < col_ncl[c]; ++k) cl_col[first + k] = c;
}

// atom of global rank g goes to its column's cluster block, in rank order;
// each system's clusters start at its fixed offset cl_off
__global__ void k_finish_perm(const int *__restrict__ tmp, const int *__restrict__ key, int n,
                              const SysDev *__restrict__ sys, const int *__restrict__ atom_sys,
                              const int *__restrict__ start,
                              const int *__restrict__ col_cl_start, int *__restrict__ perm,
                              int *__restrict__ inv_perm, const float *__restrict__ charge,
                              const float4 *__restrict__ lj, float *__restrict__ q_sorted,
                              float2 *__restrict__ prm_sorted) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const int i = tmp[g];
    const SysDev &d = sys[atom_sys[i]];
    const int lcr = (key[i] - d.key_off) / d.nzb;
    const int c = d.col_off + lcr;
    const int slot = kCluster * (d.cl_off + col_cl_start[c] - col_cl_start[d.col_off]) +
                     (g - start[d.key_off + lcr * d.nzb]);
    perm[slot] = i;
    inv_perm[i] = slot;
    q_sorted[slot] = charge[i];
    const float4 p = lj[i];
    prm_sorted[slot] = make_float2(p.x, p.y);
}

// partners in sorted indices, bit 30 kept as the 1-4 flag: the pair kernel
// masks 1-2, 1-3 and 1-4 pairs alike (1-4 pairs are evaluated by the
// special-pair kernel with their own LJ parameters); the bare-Coulomb kernel
// skips only the unflagged (1-2/1-3) partners
__global__ void k_partners_sorted(const int *__restrict__ perm, const int *__restrict__ inv_perm,
                                  const int *__restrict__ partners, int pw, int n_clusters,
                                  int *__restrict__ partners_sorted, int2 *__restrict__ range) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= n_clusters) return;
    int k = warp * kCluster + lane;
    int i = perm[k];
    int lo = 0x7fffffff, hi = -1;
    for (int w = 0; w < pw; ++w) {
        int p = -1;
        int flag = 0;
        if (i >= 0) {
            int raw = partners[(size_t)i * pw + w];
            if (raw >= 0) {
                p = inv_perm[raw & 0x3fffffff];
                flag = raw & 0x40000000;
            }
        }
        partners_sorted[(size_t)k * pw + w] = p < 0 ? -1 : (p | flag);
        if (p >= 0) {
            lo = min(lo, p);
            hi = max(hi, p);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) range[warp] = make_int2(lo, hi);
}

// one warp per cluster: FP32 coordinates + scaled charge, bounding box, and
// zeroing of the cluster's fixed-point force slots for the coming evaluation
__global__ void k_pack(PackArgs a) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= a.n_clusters) return;
    const int k = warp * kCluster + (threadIdx.x & 31);
    const int i = a.perm[k];
    double c[3] = {0.0, 0.0, 0.0};
    if (i >= 0)
        for (int d = 0; d < 3; ++d) c[d] = a.x[3 * i + d];
    pack_cluster(a, warp, k, i >= 0, c);
}

inline unsigned spread2(unsigned v) {
    v &= 0xffff;
    v = (v | (v << 8)) & 0x00FF00FF;
    v = (v | (v << 4)) & 0x0F0F0F0F;
    v = (v | (v << 2)) & 0x33333333;
    v = (v | (v << 1)) & 0x55555555;
    return v;
}

template <typename T>
int realloc_dev(T **p, size_t count) {
    cudaFree(*p);
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, count * sizeof(T)) == cudaSuccess ? MDG_OK : MDG_ERR_NOMEM;
}

}  // namespace

// host: column grid of every system (box and density), the system table,
// and every buffer whose size depends on them (the cluster-order arrays are
// sized for the worst-case padding: one partial cluster per column)
int prepare_sort_grid(mdg_system *s) {
    std::vector<int> col_rank_all, col_sys, cl_sys, col_xy;
    int col_off = 0, key_off = 0, cl_off = 0;
    for (int q = 0; q < s->n_sys; ++q) {
        SysDev &d = s->sys_h[q];
        const double V = d.Ld[0] * d.Ld[1] * d.Ld[2];
        const double rho = std::max(d.n_atoms / V, 1e-6);
        const double a = std::cbrt((double)kCluster / rho);
        d.ncx = std::max(1, std::min(4096, (int)std::lround(d.Ld[0] / a)));
        d.ncy = std::max(1, std::min(4096, (int)std::lround(d.Ld[1] / a)));
        d.nzb = std::max(1, std::min(8192, (int)std::lround(d.Ld[2] / (a / 8.0))));
        d.n_cols = d.ncx * d.ncy;
        d.col_off = col_off;
        d.key_off = key_off;
        d.cl_off = cl_off;
        d.cl_cap = (d.n_atoms + kCluster - 1) / kCluster + d.n_cols;
        std::vector<std::pair<unsigned, int>> codes(d.n_cols);
        for (int cx = 0; cx < d.ncx; ++cx)
            for (int cy = 0; cy < d.ncy; ++cy)
                codes[cx * d.ncy + cy] = {spread2(cx) | (spread2(cy) << 1), cx * d.ncy + cy};
        std::sort(codes.begin(), codes.end());
        std::vector<int> rank(d.n_cols), xy(d.n_cols);
        for (int r = 0; r < d.n_cols; ++r) {
            const int cxy = codes[r].second;
            rank[cxy] = r;
            xy[r] = ((cxy / d.ncy) << 16) | (cxy % d.ncy);
        }
        // neighbour-column pair search needs at least 5 columns per axis
        // (whether the reach fits is decided on the device every step)
        d.col_mode = (d.ncx >= 5 && d.ncy >= 5) ? 1 : 0;
        col_xy.insert(col_xy.end(), xy.begin(), xy.end());
        col_rank_all.insert(col_rank_all.end(), rank.begin(), rank.end());
        col_sys.insert(col_sys.end(), d.n_cols, q);
        cl_sys.insert(cl_sys.end(), d.cl_cap, q);
        col_off += d.n_cols;
        if ((long long)key_off + (long long)d.n_cols * d.nzb > (1ll << 28)) return MDG_ERR_INVALID;
        key_off += d.n_cols * d.nzb;
        cl_off += d.cl_cap;
    }
    s->n_cols = col_off;
    s->n_cells = key_off;
    s->n_scan_blocks = (int)(((long long)key_off + kScanPerBlock - 1) / kScanPerBlock);
    const int n_clusters = cl_off;
    const int n_pad = n_clusters * kCluster;
    int rc = MDG_OK;
    if ((rc = realloc_dev(&s->cell_rank, col_off)) || (rc = realloc_dev(&s->cell_count, key_off)) ||
        (rc = realloc_dev(&s->cell_start, (size_t)key_off + 1)) ||
        (rc = realloc_dev(&s->cell_cursor, key_off)) ||
        (rc = realloc_dev(&s->scan_blocks, s->n_scan_blocks)) ||
        (rc = realloc_dev(&s->col_ncl, col_off)) || (rc = realloc_dev(&s->col_cl_start, col_off + 1)) ||
        (rc = realloc_dev(&s->col_sys, col_off)) || (rc = realloc_dev(&s->col_xy, col_off)) ||
        (rc = realloc_dev(&s->overhang, s->n_sys)))
        return rc;
    if (n_pad != s->n_pad || !s->perm) {
        s->n_pad = n_pad;
        s->n_clusters = n_clusters;
        if ((rc = realloc_dev(&s->perm, n_pad)) || (rc = realloc_dev(&s->q_sorted, n_pad)) ||
            (rc = realloc_dev(&s->prm_sorted, n_pad)) || (rc = realloc_dev(&s->xq, n_pad)) ||
            (rc = realloc_dev(&s->f, 3 * (size_t)n_pad)) ||
            (rc = realloc_dev(&s->bbox, 2 * (size_t)n_clusters)) ||
            (rc = realloc_dev(&s->hbox, 4 * (size_t)n_clusters)) ||
            (rc = realloc_dev(&s->qbox, 8 * (size_t)n_clusters)) ||
            (rc = realloc_dev(&s->cluster_partner_range, n_clusters)) ||
            (rc = realloc_dev(&s->cl_sys, n_clusters)) ||
            (rc = realloc_dev(&s->cl_col, n_clusters)) ||
            (rc = realloc_dev(&s->partners_sorted, (size_t)n_pad * std::max(s->pw, 1))))
            return rc;
        if (cudaMemset(s->f, 0, sizeof(unsigned long long) * 3 * n_pad) != cudaSuccess)
            return MDG_ERR_CUDA;
    }
    if (cudaMemcpy(s->cell_rank, col_rank_all.data(), sizeof(int) * col_off,
                   cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->col_sys, col_sys.data(), sizeof(int) * col_off, cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(s->col_xy, col_xy.data(), sizeof(int) * col_off, cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(s->cl_sys, cl_sys.data(), sizeof(int) * n_clusters, cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return MDG_ERR_CUDA;
    return upload_sys_table(s);
}

int upload_sys_table(mdg_system *s) {
    if (!s->sys_dev && cudaMalloc(&s->sys_dev, sizeof(SysDev) * s->n_sys) != cudaSuccess)
        return MDG_ERR_NOMEM;
    return cudaMemcpy(s->sys_dev, s->sys_h.data(), sizeof(SysDev) * s->n_sys,
                      cudaMemcpyHostToDevice) == cudaSuccess
               ? MDG_OK
               : MDG_ERR_CUDA;
}

cudaError_t launch_reorder(mdg_system *s) {
    cudaStream_t st = s->stream;
    const int n = s->n;
    const int tb = 256;
    cudaMemsetAsync(s->cell_count, 0, sizeof(int) * s->n_cells, st);
    cudaMemsetAsync(s->cell_cursor, 0, sizeof(int) * s->n_cells, st);
    cudaMemsetAsync(s->perm, 0xff, sizeof(int) * s->n_pad, st);
    cudaMemsetAsync(s->q_sorted, 0, sizeof(float) * s->n_pad, st);
    cudaMemsetAsync(s->prm_sorted, 0, sizeof(float2) * s->n_pad, st);
    cudaMemsetAsync(s->cl_col, 0xff, sizeof(int) * s->n_clusters, st);
    cudaMemsetAsync(s->overhang, 0, sizeof(float) * s->n_sys, st);
    k_bin<<<(n + tb - 1) / tb, tb, 0, st>>>(s->x, n, s->sys_dev, s->atom_sys, s->cell_rank,
                                            s->atom_key, s->cell_count, s->status);
    k_block_sums<<<s->n_scan_blocks, kScanThreads, 0, st>>>(s->cell_count, s->n_cells,
                                                            s->scan_blocks);
    k_scan_top<<<1, kScanThreads, 0, st>>>(s->scan_blocks, s->n_scan_blocks);
    k_scan_final<<<s->n_scan_blocks, kScanThreads, 0, st>>>(s->cell_count, s->n_cells,
                                                            s->scan_blocks, s->cell_start);
    k_col_clusters<<<(s->n_cols + tb - 1) / tb, tb, 0, st>>>(s->cell_start, s->n_cols,
                                                             s->sys_dev, s->col_sys, s->col_ncl);
    k_col_scan<<<1, kScanThreads, 0, st>>>(s->col_ncl, s->n_cols, s->col_cl_start);
    k_cluster_columns<<<(s->n_cols + tb - 1) / tb, tb, 0, st>>>(s->col_ncl, s->col_cl_start,
                                                                s->n_cols, s->sys_dev, s->col_sys,
                                                                s->cl_col);
    k_scatter<<<(n + tb - 1) / tb, tb, 0, st>>>(s->atom_key, n, s->cell_start, s->cell_cursor,
                                                s->tmp_perm);
    k_cell_sort<<<(s->n_cells + tb - 1) / tb, tb, 0, st>>>(s->cell_start, s->n_cells, s->tmp_perm);
    k_finish_perm<<<(n + tb - 1) / tb, tb, 0, st>>>(s->tmp_perm, s->atom_key, n, s->sys_dev,
                                                    s->atom_sys, s->cell_start, s->col_cl_start,
                                                    s->perm,
                                                    s->inv_perm, s->charge, s->lj, s->q_sorted,
                                                    s->prm_sorted);
    k_partners_sorted<<<(s->n_clusters * 32 + tb - 1) / tb, tb, 0, st>>>(
        s->perm, s->inv_perm, s->partners, s->pw, s->n_clusters, s->partners_sorted,
        s->cluster_partner_range);
    s->launches += 11;
    return cudaGetLastError();
}

PackArgs make_pack_args(mdg_system *s) {
    PackArgs a;
    a.x = s->x;
    a.perm = s->perm;
    a.q_sorted = s->q_sorted;
    a.n_clusters = s->n_clusters;
    a.n_pad = s->n_pad;
    a.xq = s->xq;
    a.bbox = s->bbox;
    a.hbox = s->hbox;
    a.qbox = s->qbox;
    a.f = s->f;
    a.sys = s->sys_dev;
    a.cl_sys = s->cl_sys;
    a.cl_col = s->cl_col;
    a.col_xy = s->col_xy;
    a.overhang = s->overhang;
    return a;
}

cudaError_t launch_pack(mdg_system *s) {
    const int tb = 256;
    k_pack<<<(s->n_clusters * 32 + tb - 1) / tb, tb, 0, s->stream>>>(make_pack_args(s));
    s->launches += 1;
    return cudaGetLastError();
}

}  // namespace mdg
