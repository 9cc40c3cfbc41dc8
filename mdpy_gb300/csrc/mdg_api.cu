// mdg_api.cu -- the extern "C" entry points of libmdg (declared in include/mdg.h)
// and the orchestration of one force evaluation / MD step.
//
// One force evaluation (Ensemble.update, mdpy/ensemble.py:53-61):
//   [reorder]  spatial re-sort (every reorder_interval steps)
//   pack       FP32 cluster coordinates, bounding boxes, zeroed force slots
//   nonbonded  LJ + Ewald real space (or LJ + bare Coulomb), half shell
//   special    1-4 pairs and the Ewald exclusion correction
//   pme        spread -> R2C -> convolve -> C2R -> gather
//   bonded     bonds, angles, dihedrals, impropers
// One MD step (Integrator.integrate, one step): pre-force update, force
// evaluation, post-force update.  mdg_integrate replays chunks of
// `reorder_interval` steps as one CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mdg_internal.cuh"

using namespace mdg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    return fail(e == cudaErrorMemoryAllocation ? MDG_ERR_NOMEM : MDG_ERR_CUDA, "%s: %s", where,
                cudaGetErrorString(e));
}

#define CK(call, where)                                   \
    do {                                                  \
        cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return cuda_fail(_e, where); \
    } while (0)

template <typename T>
int dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    return MDG_OK;
}

template <typename T>
void dfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

int check_sys(mdg_system *s) {
    if (!s) return fail(MDG_ERR_INVALID, "null system");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return MDG_OK;
}

void drop_one(Graph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    g.steps = 0;
}

void drop_graph(mdg_system *s) {
    drop_one(s->graph);
    for (auto &plane : s->graph_step)
        for (auto &row : plane)
            for (Graph &g : row) drop_one(g);
    for (Graph &g : s->graph_eval) drop_one(g);
}

int validate_box(const double *box, double cutoff) {
    for (int d = 0; d < 3; ++d) {
        if (!(box[d] > 0) || !std::isfinite(box[d]))
            return fail(MDG_ERR_BOX, "box edge %d is %g; edges must be positive", d, box[d]);
        if (cutoff > 0 && !(cutoff < 0.5 * box[d]))
            return fail(MDG_ERR_CUTOFF,
                        "cutoff %g must be below half the box edge %g (minimum image)", cutoff,
                        box[d]);
    }
    return MDG_OK;
}

int validate_boxes(mdg_system *s, double cutoff) {
    for (const SysDev &d : s->sys_h) {
        const int rc = validate_box(d.Ld, cutoff);
        if (rc) return rc;
    }
    return MDG_OK;
}

void set_sys_box(SysDev &d, const double *box) {
    for (int k = 0; k < 3; ++k) {
        d.Ld[k] = box[k];
        d.invLd[k] = 1.0 / box[k];
        d.L[k] = (float)box[k];
        d.invL[k] = (float)(1.0 / box[k]);
    }
}

double coulomb_k() {
    // k_e = 1/(4 pi eps0) from mdpy's constants (mdpy/unit/__init__.py:56-58)
    const double eps0 = 8.85418e-12 * 1.66053904e-27 / (1.602176634e-19 * 1.602176634e-19);
    return 1.0 / (4.0 * 3.14159265358979323846 * eps0);
}

// FP64 Ewald self and net-charge energies of every system (depend on the
// charges, beta and the box volume)
void ewald_constants(mdg_system *s) {
    const double ke = coulomb_k(), pi = 3.14159265358979323846, b = s->pme.beta;
    s->e_self.assign(s->n_sys, 0.0);
    s->e_net.assign(s->n_sys, 0.0);
    if (!(b > 0)) return;
    for (int q = 0; q < s->n_sys; ++q) {
        const double *L = s->sys_h[q].Ld;
        const double V = L[0] * L[1] * L[2];
        s->e_self[q] = -ke * b / std::sqrt(pi) * s->q2sum[q];
        s->e_net[q] = -ke * pi * s->qsum[q] * s->qsum[q] / (2.0 * b * b * V);
    }
}

int decode_status(mdg_system *s, int st) {
    if (st) {
        CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
        for (int code = 1; code < 31; ++code)
            if (st & (1 << code)) {
                switch (code) {
                    case MDG_ERR_PARTICLE_LOSS:
                        return fail(code, "non-finite position or velocity, or a position two "
                                          "or more box lengths from the central image");
                    case MDG_ERR_OVERFLOW:
                        return fail(code, "force or energy beyond the int64 fixed-point range");
                    default:
                        return fail(code, "device status %d", code);
                }
            }
    }
    return MDG_OK;
}

int read_status(mdg_system *s) {
    int st = 0;
    CK(cudaMemcpyAsync(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream),
       "status read");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return decode_status(s, st);
}

int evaluate(mdg_system *s, unsigned mask, int energy) {
    if (s->need_reorder) {
        CK(launch_reorder(s), "reorder");
        s->need_reorder = 0;
        s->steps_since_reorder = 0;
    }
    if (energy) {
        CK(cudaMemsetAsync(s->energy, 0, sizeof(long long) * kEnergySlots * s->n_sys, s->stream),
           "memset");
        CK(cudaMemsetAsync(s->stats, 0, sizeof(unsigned long long) * 4, s->stream), "memset");
    }
    CK(launch_pack(s), "pack");
    const int lsp = s->ls ? s->ls_phase : kLsOff;
    if (lsp >= kLsOuter)  // full evaluation of the learned form: slow force kept apart
        CK(cudaMemsetAsync(s->ls->fs, 0, sizeof(unsigned long long) * 3 * (size_t)s->n_pad,
                           s->stream),
           "memset");
    // fork: PME on one side stream, special pairs and bonded terms on
    // another, while the pair kernel runs on the main stream (all accumulate
    // through order-independent fixed-point atomics); join both before
    // anything reads f
    CK(cudaEventRecord(s->ev_fork, s->stream), "fork");
    CK(cudaStreamWaitEvent(s->side_stream, s->ev_fork, 0), "fork wait");
    CK(cudaStreamWaitEvent(s->bond_stream, s->ev_fork, 0), "fork wait");
    cudaStream_t main = s->stream;
    int rc = MDG_OK;
    cudaError_t e = cudaSuccess;
    s->stream = s->side_stream;
    // (multiple time steps: weight 0 leaves the reciprocal force out, and the
    // term runs at all only when its energy is wanted)
    if (s->recip_weight == 0.f && !energy) mask &= ~MDG_MASK(MDG_TERM_COUL_RECIP);
    if ((mask & MDG_MASK(MDG_TERM_COUL_RECIP)) && s->pme.on) {
        int cr = 0;
        e = launch_pme(s, energy, &cr);
        if (cr != CUFFT_SUCCESS) rc = fail(MDG_ERR_CUFFT, "cuFFT execution failed (%d)", cr);
    }
    // learned slow force: features and MLP after PME on the same stream
    if (!rc && e == cudaSuccess && lsp != kLsOff) e = ls_side(s, lsp);
    cudaError_t ej = cudaEventRecord(s->ev_join, s->side_stream);
    s->stream = s->bond_stream;
    if (!rc && e == cudaSuccess) e = launch_special(s, mask, energy, 0);
    if (!rc && e == cudaSuccess) e = launch_bonded(s, mask, energy);
    cudaError_t ej2 = cudaEventRecord(s->ev_join2, s->bond_stream);
    s->stream = main;
    if (rc) return rc;
    CK(e, "side-stream terms");
    CK(ej, "join");
    CK(ej2, "join");
    CK(launch_nonbonded(s, mask, energy, 0), "nonbonded");
    CK(cudaStreamWaitEvent(s->stream, s->ev_join, 0), "join wait");
    CK(cudaStreamWaitEvent(s->stream, s->ev_join2, 0), "join wait");
    if (lsp != kLsOff) CK(ls_after_join(s, lsp), "learned slow force");
    s->evaluated_once = 1;
    return MDG_OK;
}

bool ls_active(const mdg_system *s) { return s->ls && s->ls->enabled; }

// One evaluation of the learned form (phase kLsInner / kLsOuter / kLsAnchor):
// PME only at full evaluations, into the slow-force buffer.
int ls_evaluate(mdg_system *s, unsigned mask, int energy, int phase) {
    const bool full = phase != kLsInner;
    s->ls_phase = phase;
    s->recip_weight = full ? 1.0f : 0.0f;
    s->slow_target = full ? s->ls->fs : nullptr;
    const int rc = evaluate(s, mask, energy);
    s->ls_phase = kLsOff;
    s->slow_target = nullptr;
    s->recip_weight = 1.0f;
    s->forces_weight = -1.0f;
    return rc;
}

// weight of the reciprocal force in the evaluation that ends step `step`:
// mts_k at the end of an outer step of the multiple-time-step scheme, else 0
float mts_weight(const mdg_system *s, uint64_t step) {
    if (s->mts_k <= 1) return 1.0f;
    return ((step + 1) % (uint64_t)s->mts_k == 0) ? (float)s->mts_k : 0.0f;
}

int md_step(mdg_system *s, unsigned mask, int energy) {
    // (the pre-force update stays its own coalesced pass over atom order: a
    // version fused into the cluster-order packing measured 1 % slower)
    CK(launch_integrate_pre(s), "integrate pre");
    if (s->steps_since_reorder >= s->reorder_interval) s->need_reorder = 1;
    int rc;
    if (ls_active(s)) {
        rc = ls_evaluate(s, mask, energy, mts_weight(s, s->step) != 0.f ? kLsOuter : kLsInner);
    } else {
        s->recip_weight = mts_weight(s, s->step);
        rc = evaluate(s, mask, energy);
        s->forces_weight = s->recip_weight;
        s->recip_weight = 1.0f;
    }
    if (rc) return rc;
    CK(launch_integrate_post(s, energy), "integrate post");
    s->steps_since_reorder += 1;
    s->step += 1;
    return MDG_OK;
}

// Capture `nsteps` MD steps (the first re-sorting the atoms when `resort`)
// into g; host-side counters are restored, the launch count per replay is
// kept in g.steps.
int capture_steps(mdg_system *s, Graph &g, int nsteps, int resort, unsigned mask,
                  int energy_last = 0) {
    const long long saved = s->launches;
    const int saved_since = s->steps_since_reorder, saved_need = s->need_reorder;
    const uint64_t saved_step = s->step;
    s->need_reorder = resort ? 1 : 0;
    if (!resort) s->steps_since_reorder = 0;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "capture");
    int crc = MDG_OK;
    for (int k = 0; k < nsteps && !crc; ++k)
        crc = md_step(s, mask, (energy_last && k == nsteps - 1) ? 1 : 0);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s->stream, &graph);
    s->steps_since_reorder = saved_since;
    s->need_reorder = saved_need;
    s->step = saved_step;
    const long long per = s->launches - saved;
    s->launches = saved;
    if (crc) {
        if (graph) cudaGraphDestroy(graph);
        return crc;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "end capture");
    ce = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        g.exec = nullptr;
        return cuda_fail(ce, "graph instantiate");
    }
    g.steps = (int)per;
    g.mask = mask;
    return MDG_OK;
}

// The force evaluation an integration starts with when the forces are not
// valid (new positions): captured once per re-sort flag and replayed.
int capture_eval(mdg_system *s, Graph &g, int resort, unsigned mask) {
    const long long saved = s->launches;
    const int saved_need = s->need_reorder, saved_since = s->steps_since_reorder;
    s->need_reorder = resort ? 1 : 0;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "capture");
    const int crc = evaluate(s, mask, 0);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s->stream, &graph);
    s->need_reorder = saved_need;
    s->steps_since_reorder = saved_since;
    const long long per = s->launches - saved;
    s->launches = saved;
    if (crc) {
        if (graph) cudaGraphDestroy(graph);
        return crc;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "end capture");
    ce = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        g.exec = nullptr;
        return cuda_fail(ce, "graph instantiate");
    }
    g.steps = (int)per;
    g.mask = mask;
    return MDG_OK;
}

int ready_for_forces(mdg_system *s, unsigned mask) {
    if (!s->have_x) return fail(MDG_ERR_STATE, "positions have not been set");
    if ((mask & (MDG_MASK(MDG_TERM_LJ) | MDG_MASK(MDG_TERM_COUL_REAL))) && !s->nb_configured)
        return fail(MDG_ERR_STATE, "nonbonded terms requested but not configured");
    if ((mask & MDG_MASK(MDG_TERM_LJ)) && s->lj_on && !s->have_lj)
        return fail(MDG_ERR_STATE, "LJ parameters have not been set");
    if ((mask & (MDG_MASK(MDG_TERM_COUL_REAL) | MDG_MASK(MDG_TERM_COUL_RECIP))) &&
        !s->have_charges)
        return fail(MDG_ERR_STATE, "charges have not been set");
    return MDG_OK;
}

}  // namespace

extern "C" {

MDG_API int mdg_version(int *major, int *minor) {
    if (major) *major = 1;
    if (minor) *minor = 0;
    return MDG_OK;
}

MDG_API const char *mdg_last_error(void) { return g_last_error.c_str(); }

MDG_API int mdg_system_create(int device, int n_atoms, const double *box, mdg_system **out) {
    return mdg_system_create_batch(device, 1, &n_atoms, box, out);
}

MDG_API int mdg_system_create_batch(int device, int n_systems, const int *n_atoms,
                                    const double *boxes, mdg_system **out) {
    if (!out) return fail(MDG_ERR_INVALID, "out is null");
    *out = nullptr;
    if (n_systems < 1 || n_systems > 65536)
        return fail(MDG_ERR_INVALID, "n_systems %d out of range", n_systems);
    if (!n_atoms || !boxes) return fail(MDG_ERR_INVALID, "n_atoms or boxes is null");
    long long total = 0;
    for (int q = 0; q < n_systems; ++q) {
        if (n_atoms[q] <= 0 || n_atoms[q] > (1 << 26))
            return fail(MDG_ERR_INVALID, "n_atoms %d of system %d out of range", n_atoms[q], q);
        total += n_atoms[q];
        int rc = validate_box(boxes + 3 * q, 0.0);
        if (rc) return rc;
    }
    if (total > (1 << 26)) return fail(MDG_ERR_INVALID, "%lld atoms in total: too many", total);
    CK(cudaSetDevice(device), "cudaSetDevice");
    mdg_system *s = new mdg_system();
    s->device = device;
    s->n = (int)total;
    s->n_sys = n_systems;
    s->sys_h.assign(n_systems, SysDev{});
    s->atoms_per_sys.assign(n_atoms, n_atoms + n_systems);
    s->qsum.assign(n_systems, 0.0);
    s->q2sum.assign(n_systems, 0.0);
    s->e_self.assign(n_systems, 0.0);
    s->e_net.assign(n_systems, 0.0);
    std::vector<int> atom_sys(total);
    int off = 0;
    for (int q = 0; q < n_systems; ++q) {
        SysDev &d = s->sys_h[q];
        set_sys_box(d, boxes + 3 * q);
        d.atom_off = off;
        d.n_atoms = n_atoms[q];
        std::fill(atom_sys.begin() + off, atom_sys.begin() + off + n_atoms[q], q);
        off += n_atoms[q];
    }
    cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaStreamCreate");
    }
    s->stream = s->own_stream;
    {
        // two side streams: normal priority, and the highest priority (its
        // small kernels then take free SM slots ahead of the pair kernel's
        // queued CTAs); the launch shape picks one
        int lo = 0, hi = 0;
        e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = cudaStreamCreateWithPriority(&s->side_streams[k], cudaStreamNonBlocking,
                                             k ? hi : lo);
            if (e == cudaSuccess)
                e = cudaStreamCreateWithPriority(&s->bond_streams[k], cudaStreamNonBlocking,
                                                 k ? hi : lo);
        }
        s->side_stream = s->side_streams[0];
        s->bond_stream = s->bond_streams[0];
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join2, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        mdg_system_destroy(s);
        return cuda_fail(e, "side stream");
    }
    const int n = s->n;
    int rc = MDG_OK;
#define AL(ptr, cnt)                     \
    if ((rc = dalloc(&(ptr), (cnt)))) { \
        mdg_system_destroy(s);          \
        return rc;                      \
    }
    AL(s->mass, n);
    AL(s->inv_mass, n);
    AL(s->charge, n);
    AL(s->lj, n);
    AL(s->inv_perm, n);
    AL(s->atom_key, n);
    AL(s->tmp_perm, n);
    AL(s->atom_sys, n);
    AL(s->x, 3 * (size_t)n);
    AL(s->v, 3 * (size_t)n);
    AL(s->energy, (size_t)kEnergySlots * n_systems);
    AL(s->status, 1);
    AL(s->stats, 4);
    AL(s->step_dev, 1);
    AL(s->fout, 3 * (size_t)n);
    AL(s->dump_count, 1);
    AL(s->partners, 1);
    AL(s->nb_queue, 1);
#undef AL
    {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        s->n_sms = std::max(1, sms);
    }
    cudaMemset(s->energy, 0, sizeof(long long) * kEnergySlots * n_systems);
    cudaMemset(s->status, 0, sizeof(int));
    cudaMemset(s->step_dev, 0, sizeof(unsigned long long));
    cudaMemset(s->v, 0, sizeof(double) * 3 * n);
    cudaMemset(s->lj, 0, sizeof(float4) * n);
    cudaMemset(s->charge, 0, sizeof(float) * n);
    cudaMemcpy(s->atom_sys, atom_sys.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    // masses default to 1 (inv 1) so kinetic terms are defined before set_masses
    std::vector<double> ones(n, 1.0);
    cudaMemcpy(s->mass, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(s->inv_mass, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    s->pw = 0;
    rc = prepare_sort_grid(s);
    if (rc) {
        mdg_system_destroy(s);
        return fail(rc, "sort grid allocation failed");
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        mdg_system_destroy(s);
        return cuda_fail(e, "system create");
    }
    *out = s;
    return MDG_OK;
}

MDG_API int mdg_num_systems(mdg_system *s, int *n_systems) {
    if (!s || !n_systems) return fail(MDG_ERR_INVALID, "null argument");
    *n_systems = s->n_sys;
    return MDG_OK;
}

MDG_API int mdg_system_destroy(mdg_system *s) {
    if (!s) return MDG_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    drop_graph(s);
    pme_free(s);
    dfree(s->mass);
    dfree(s->inv_mass);
    dfree(s->charge);
    dfree(s->lj);
    dfree(s->partners);
    dfree(s->excl_pairs);
    dfree(s->pairs14);
    dfree(s->perm);
    dfree(s->inv_perm);
    dfree(s->q_sorted);
    dfree(s->prm_sorted);
    dfree(s->partners_sorted);
    dfree(s->cluster_partner_range);
    dfree(s->cell_rank);
    dfree(s->cell_count);
    dfree(s->cell_start);
    dfree(s->cell_cursor);
    dfree(s->atom_key);
    dfree(s->tmp_perm);
    dfree(s->atom_sys);
    dfree(s->cl_sys);
    dfree(s->col_sys);
    dfree(s->cl_col);
    dfree(s->nb_queue);
    dfree(s->col_xy);
    dfree(s->overhang);
    dfree(s->sys_dev);
    dfree(s->scan_blocks);
    dfree(s->col_ncl);
    dfree(s->col_cl_start);
    dfree(s->x);
    dfree(s->v);
    dfree(s->f);
    dfree(s->xq);
    dfree(s->bbox);
    dfree(s->hbox);
    dfree(s->qbox);
    dfree(s->energy);
    dfree(s->status);
    dfree(s->stats);
    dfree(s->step_dev);
    dfree(s->fout);
    dfree(s->dump_count);
    dfree(s->bond_idx);
    dfree(s->bond_prm);
    dfree(s->angle_idx);
    dfree(s->angle_prm);
    dfree(s->dih_idx);
    dfree(s->dih_prm);
    dfree(s->imp_idx);
    dfree(s->imp_prm);
    ls_free(s);
    for (cudaStream_t *pair : {s->side_streams, s->bond_streams})
        for (int k = 0; k < 2; ++k)
            if (pair[k]) {
                cudaStreamSynchronize(pair[k]);
                cudaStreamDestroy(pair[k]);
            }
    if (s->ev_join2) cudaEventDestroy(s->ev_join2);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    if (s->host_stage) cudaFreeHost(s->host_stage);
    for (cudaEvent_t &ev : s->snap_ev)
        if (ev) cudaEventDestroy(ev);
    if (s->snap_host) cudaFreeHost(s->snap_host);
    dfree(s->xin);
    dfree(s->vsave);
    dfree(s->same_flag);
    delete s;
    return MDG_OK;
}

MDG_API int mdg_system_set_stream(mdg_system *s, void *stream) {
    int rc = check_sys(s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    s->stream = stream ? (cudaStream_t)stream : s->own_stream;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_system_set_box(mdg_system *s, const double *box) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!box) return fail(MDG_ERR_INVALID, "box is null");
    std::vector<double> all(3 * (size_t)s->n_sys);
    for (int q = 0; q < s->n_sys; ++q) std::copy(box, box + 3, all.begin() + 3 * q);
    return mdg_system_set_boxes(s, all.data());
}

MDG_API int mdg_system_set_boxes(mdg_system *s, const double *boxes) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!boxes) return fail(MDG_ERR_INVALID, "boxes is null");
    for (int q = 0; q < s->n_sys; ++q) {
        rc = validate_box(boxes + 3 * q, s->nb_configured ? s->cutoff : 0.0);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    for (int q = 0; q < s->n_sys; ++q) set_sys_box(s->sys_h[q], boxes + 3 * q);
    rc = prepare_sort_grid(s);
    if (rc) return fail(rc, "sort grid allocation failed");
    if (s->pme.on) {
        std::vector<int> grids(3 * (size_t)s->n_sys);
        for (int q = 0; q < s->n_sys; ++q)
            for (int d = 0; d < 3; ++d) grids[3 * q + d] = s->sys_h[q].K[d];
        rc = pme_setup(s, grids.data());
        if (rc) return fail(rc, "PME set-up failed");
        ewald_constants(s);
    }
    if (s->ls) {  // the learned form's cell grid follows the box (parameters kept)
        const Learned &L = *s->ls;
        const int on = L.enabled, k = L.k, tc = L.use_tc, cap = L.cap;
        const int ty = L.use_taylor, nt = L.use_net;
        const float thr = L.threshold, rf = L.rf, skin = L.skin;
        rc = ls_configure(s, rf, skin, cap);
        if (rc) return fail(rc, "learned slow force: box too small or allocation failed");
        s->ls->use_taylor = ty;
        s->ls->use_net = nt;
        s->ls->enabled = on;
        s->ls->k = k;
        s->ls->threshold = thr;
        s->ls->use_tc = tc;
    }
    s->need_reorder = 1;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_set_masses(mdg_system *s, const double *m) {
    int rc = check_sys(s);
    if (rc) return rc;
    std::vector<double> mm(m, m + s->n), inv(s->n);
    for (int i = 0; i < s->n; ++i) {
        if (!(mm[i] > 0)) return fail(MDG_ERR_INVALID, "mass of atom %d is %g", i, mm[i]);
        inv[i] = 1.0 / mm[i];
    }
    CK(cudaMemcpy(s->mass, mm.data(), sizeof(double) * s->n, cudaMemcpyHostToDevice), "copy");
    CK(cudaMemcpy(s->inv_mass, inv.data(), sizeof(double) * s->n, cudaMemcpyHostToDevice), "copy");
    s->have_masses = 1;
    return MDG_OK;
}

MDG_API int mdg_set_charges(mdg_system *s, const double *q_in) {
    int rc = check_sys(s);
    if (rc) return rc;
    // q * sqrt(k_e), k_e = 1/(4 pi eps0) from mdpy's constants
    const double sk = std::sqrt(coulomb_k());
    std::vector<float> qs(s->n);
    for (int q = 0; q < s->n_sys; ++q) {
        const SysDev &d = s->sys_h[q];
        double sum = 0.0, sum2 = 0.0;
        for (int i = d.atom_off; i < d.atom_off + d.n_atoms; ++i) {
            qs[i] = (float)(q_in[i] * sk);
            sum += q_in[i];
            sum2 += q_in[i] * q_in[i];
        }
        s->qsum[q] = sum;
        s->q2sum[q] = sum2;
    }
    CK(cudaMemcpy(s->charge, qs.data(), sizeof(float) * s->n, cudaMemcpyHostToDevice), "copy");
    s->have_charges = 1;
    s->need_reorder = 1;
    s->forces_valid = 0;
    drop_graph(s);
    ewald_constants(s);  // the FP64 Ewald constants depend on the charges
    return MDG_OK;
}

MDG_API int mdg_set_lj(mdg_system *s, const double *params) {
    int rc = check_sys(s);
    if (rc) return rc;
    std::vector<float4> p(s->n);
    for (int i = 0; i < s->n; ++i) {
        const double *r = params + 4 * i;
        if (r[0] < 0 || r[2] < 0) return fail(MDG_ERR_INVALID, "negative epsilon for atom %d", i);
        p[i] = make_float4((float)(0.5 * r[1]), (float)std::sqrt(4.0 * r[0]), (float)(0.5 * r[3]),
                           (float)std::sqrt(4.0 * r[2]));
    }
    CK(cudaMemcpy(s->lj, p.data(), sizeof(float4) * s->n, cudaMemcpyHostToDevice), "copy");
    s->have_lj = 1;
    s->need_reorder = 1;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_set_exclusions(mdg_system *s, const int32_t *bonded, int bw,
                               const int32_t *scaling, int sw) {
    int rc = check_sys(s);
    if (rc) return rc;
    const int n = s->n;
    if (bw < 0 || sw < 0) return fail(MDG_ERR_INVALID, "negative width");
    // symmetric partner sets; a pair listed as both 1-2/1-3 and 1-4 stays excluded
    std::vector<std::vector<int>> excl(n), p14(n);
    std::vector<int> sys_of(n);
    for (int q = 0; q < s->n_sys; ++q)
        std::fill(sys_of.begin() + s->sys_h[q].atom_off,
                  sys_of.begin() + s->sys_h[q].atom_off + s->sys_h[q].n_atoms, q);
    auto add = [&](std::vector<std::vector<int>> &lst, int i, int j) {
        if (j < 0) return 0;
        if (j >= n || j == i || sys_of[j] != sys_of[i]) return 1;
        if (std::find(lst[i].begin(), lst[i].end(), j) == lst[i].end()) lst[i].push_back(j);
        if (std::find(lst[j].begin(), lst[j].end(), i) == lst[j].end()) lst[j].push_back(i);
        return 0;
    };
    for (int i = 0; i < n; ++i) {
        for (int w = 0; w < bw; ++w)
            if (add(excl, i, bonded[(size_t)i * bw + w]))
                return fail(MDG_ERR_INVALID, "bad bonded partner of atom %d", i);
        for (int w = 0; w < sw; ++w)
            if (add(p14, i, scaling[(size_t)i * sw + w]))
                return fail(MDG_ERR_INVALID, "bad 1-4 partner of atom %d", i);
    }
    int pw = 0;
    std::vector<int2> ex, s14;
    for (int i = 0; i < n; ++i) {
        auto &e = excl[i];
        std::vector<int> p14only;
        for (int j : p14[i])
            if (std::find(e.begin(), e.end(), j) == e.end()) p14only.push_back(j);
        p14[i] = p14only;
        pw = std::max<int>(pw, (int)(e.size() + p14[i].size()));
        for (int j : e)
            if (j > i) ex.push_back(make_int2(i, j));
        for (int j : p14[i])
            if (j > i) s14.push_back(make_int2(i, j));
    }
    std::vector<int> flat((size_t)n * std::max(pw, 1), -1);
    for (int i = 0; i < n; ++i) {
        int w = 0;
        for (int j : excl[i]) flat[(size_t)i * pw + w++] = j;
        for (int j : p14[i]) flat[(size_t)i * pw + w++] = j | 0x40000000;
    }
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    dfree(s->partners);
    dfree(s->partners_sorted);
    dfree(s->excl_pairs);
    dfree(s->pairs14);
    s->pw = pw;
    if ((rc = dalloc(&s->partners, flat.size()))) return rc;
    if ((rc = dalloc(&s->partners_sorted, (size_t)s->n_pad * std::max(pw, 1)))) return rc;
    if ((rc = dalloc(&s->excl_pairs, ex.size()))) return rc;
    if ((rc = dalloc(&s->pairs14, s14.size()))) return rc;
    CK(cudaMemcpy(s->partners, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice), "copy");
    if (!ex.empty())
        CK(cudaMemcpy(s->excl_pairs, ex.data(), sizeof(int2) * ex.size(), cudaMemcpyHostToDevice), "copy");
    if (!s14.empty())
        CK(cudaMemcpy(s->pairs14, s14.data(), sizeof(int2) * s14.size(), cudaMemcpyHostToDevice), "copy");
    s->n_excl = (int)ex.size();
    s->n_14 = (int)s14.size();
    s->need_reorder = 1;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_nonbonded_config(mdg_system *s, double cutoff, double switch_radius, int lj_on,
                                 int coulomb_mode, double beta) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (coulomb_mode < MDG_COUL_NONE || coulomb_mode > MDG_COUL_BARE)
        return fail(MDG_ERR_INVALID, "unknown coulomb mode %d", coulomb_mode);
    if (!(cutoff > 0)) return fail(MDG_ERR_CUTOFF, "cutoff must be positive");
    rc = validate_boxes(s, cutoff);
    if (rc) return rc;
    if (coulomb_mode == MDG_COUL_EWALD && !(beta > 0))
        return fail(MDG_ERR_INVALID, "Ewald mode needs beta > 0");
    s->cutoff = (float)cutoff;
    s->rswitch = (switch_radius > 0 && switch_radius < cutoff) ? (float)switch_radius : 0.0f;
    s->lj_on = lj_on ? 1 : 0;
    s->coul_mode = coulomb_mode;
    s->beta = beta;
    s->nb_configured = 1;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_pme_config(mdg_system *s, const int *grid, int order, double beta) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!grid) return fail(MDG_ERR_INVALID, "grid is null");
    std::vector<int> grids(3 * (size_t)s->n_sys);
    for (int q = 0; q < s->n_sys; ++q) std::copy(grid, grid + 3, grids.begin() + 3 * q);
    return mdg_pme_config_batch(s, grids.data(), order, beta);
}

MDG_API int mdg_pme_config_batch(mdg_system *s, const int *grids, int order, double beta) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!grids) return fail(MDG_ERR_INVALID, "grids is null");
    if (order < 4 || order > 6) return fail(MDG_ERR_INVALID, "PME order %d not in 4..6", order);
    for (int t = 0; t < 3 * s->n_sys; ++t)
        if (grids[t] < 2 * order || grids[t] > 1024)
            return fail(MDG_ERR_INVALID, "PME grid %d out of range", grids[t]);
    if (!(beta > 0)) return fail(MDG_ERR_INVALID, "PME needs beta > 0");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    s->pme.order = order;
    s->pme.beta = beta;
    rc = pme_setup(s, grids);
    if (rc) {
        s->pme.on = 0;
        pme_free(s);
        return fail(rc, "PME set-up failed");
    }
    s->pme.on = 1;
    ewald_constants(s);
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_set_reorder_interval(mdg_system *s, int steps) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (steps < 1 || steps > 100000) return fail(MDG_ERR_INVALID, "interval %d out of range", steps);
    s->reorder_interval = steps;
    drop_graph(s);
    return MDG_OK;
}

static int set_terms(mdg_system *s, int n, const int32_t *idx, const double *prm, int wi, int wp,
                     int kind) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (n < 0) return fail(MDG_ERR_INVALID, "negative term count");
    for (int t = 0; t < n * wi; ++t)
        if (idx[t] < 0 || idx[t] >= s->n) return fail(MDG_ERR_INVALID, "term atom index out of range");
    if (s->n_sys > 1) {
        // a term's atoms belong to one system
        std::vector<int> sys_of(s->n);
        for (int q = 0; q < s->n_sys; ++q)
            std::fill(sys_of.begin() + s->sys_h[q].atom_off,
                      sys_of.begin() + s->sys_h[q].atom_off + s->sys_h[q].n_atoms, q);
        for (int t = 0; t < n; ++t)
            for (int k = 1; k < wi; ++k)
                if (sys_of[idx[t * wi + k]] != sys_of[idx[t * wi]])
                    return fail(MDG_ERR_INVALID, "term %d spans two systems", t);
    }
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    if (kind == 0) {
        std::vector<int2> I(n);
        std::vector<float2> P(n);
        for (int t = 0; t < n; ++t) {
            I[t] = make_int2(idx[2 * t], idx[2 * t + 1]);
            P[t] = make_float2((float)prm[2 * t], (float)prm[2 * t + 1]);
        }
        dfree(s->bond_idx);
        dfree(s->bond_prm);
        if ((rc = dalloc(&s->bond_idx, n)) || (rc = dalloc(&s->bond_prm, n))) return rc;
        if (n) {
            CK(cudaMemcpy(s->bond_idx, I.data(), sizeof(int2) * n, cudaMemcpyHostToDevice), "copy");
            CK(cudaMemcpy(s->bond_prm, P.data(), sizeof(float2) * n, cudaMemcpyHostToDevice), "copy");
        }
        s->nb = n;
    } else if (kind == 1) {
        std::vector<int4> I(n);
        std::vector<float4> P(n);
        for (int t = 0; t < n; ++t) {
            I[t] = make_int4(idx[3 * t], idx[3 * t + 1], idx[3 * t + 2], 0);
            P[t] = make_float4((float)prm[4 * t], (float)prm[4 * t + 1], (float)prm[4 * t + 2],
                               (float)prm[4 * t + 3]);
        }
        dfree(s->angle_idx);
        dfree(s->angle_prm);
        if ((rc = dalloc(&s->angle_idx, n)) || (rc = dalloc(&s->angle_prm, n))) return rc;
        if (n) {
            CK(cudaMemcpy(s->angle_idx, I.data(), sizeof(int4) * n, cudaMemcpyHostToDevice), "copy");
            CK(cudaMemcpy(s->angle_prm, P.data(), sizeof(float4) * n, cudaMemcpyHostToDevice), "copy");
        }
        s->na = n;
    } else if (kind == 2) {
        std::vector<int4> I(n);
        std::vector<float4> P(n);
        for (int t = 0; t < n; ++t) {
            I[t] = make_int4(idx[4 * t], idx[4 * t + 1], idx[4 * t + 2], idx[4 * t + 3]);
            P[t] = make_float4((float)prm[3 * t], (float)prm[3 * t + 1], (float)prm[3 * t + 2], 0.f);
        }
        dfree(s->dih_idx);
        dfree(s->dih_prm);
        if ((rc = dalloc(&s->dih_idx, n)) || (rc = dalloc(&s->dih_prm, n))) return rc;
        if (n) {
            CK(cudaMemcpy(s->dih_idx, I.data(), sizeof(int4) * n, cudaMemcpyHostToDevice), "copy");
            CK(cudaMemcpy(s->dih_prm, P.data(), sizeof(float4) * n, cudaMemcpyHostToDevice), "copy");
        }
        s->nd = n;
    } else {
        std::vector<int4> I(n);
        std::vector<float2> P(n);
        for (int t = 0; t < n; ++t) {
            I[t] = make_int4(idx[4 * t], idx[4 * t + 1], idx[4 * t + 2], idx[4 * t + 3]);
            P[t] = make_float2((float)prm[2 * t], (float)prm[2 * t + 1]);
        }
        dfree(s->imp_idx);
        dfree(s->imp_prm);
        if ((rc = dalloc(&s->imp_idx, n)) || (rc = dalloc(&s->imp_prm, n))) return rc;
        if (n) {
            CK(cudaMemcpy(s->imp_idx, I.data(), sizeof(int4) * n, cudaMemcpyHostToDevice), "copy");
            CK(cudaMemcpy(s->imp_prm, P.data(), sizeof(float2) * n, cudaMemcpyHostToDevice), "copy");
        }
        s->ni = n;
    }
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_set_bonds(mdg_system *s, int n, const int32_t *idx, const double *prm) {
    return set_terms(s, n, idx, prm, 2, 2, 0);
}
MDG_API int mdg_set_angles(mdg_system *s, int n, const int32_t *idx, const double *prm) {
    return set_terms(s, n, idx, prm, 3, 4, 1);
}
MDG_API int mdg_set_dihedrals(mdg_system *s, int n, const int32_t *idx, const double *prm) {
    return set_terms(s, n, idx, prm, 4, 3, 2);
}
MDG_API int mdg_set_impropers(mdg_system *s, int n, const int32_t *idx, const double *prm) {
    return set_terms(s, n, idx, prm, 4, 2, 3);
}

MDG_API int mdg_set_positions(mdg_system *s, const double *x, int where) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!x) return fail(MDG_ERR_INVALID, "positions pointer is null");
    CK(cudaMemcpyAsync(s->x, x, sizeof(double) * 3 * s->n,
                       where == MDG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       s->stream),
       "copy positions");
    if (where != MDG_DEVICE) CK(cudaStreamSynchronize(s->stream), "synchronize");
    s->have_x = 1;
    s->need_reorder = 1;
    s->forces_valid = 0;
    return MDG_OK;
}

MDG_API int mdg_set_velocities(mdg_system *s, const double *v, int where) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!v) return fail(MDG_ERR_INVALID, "velocities pointer is null");
    CK(cudaMemcpyAsync(s->v, v, sizeof(double) * 3 * s->n,
                       where == MDG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       s->stream),
       "copy velocities");
    if (where != MDG_DEVICE) CK(cudaStreamSynchronize(s->stream), "synchronize");
    s->have_v = 1;
    return MDG_OK;
}

MDG_API int mdg_get_positions(mdg_system *s, double *x, int where) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!x) return fail(MDG_ERR_INVALID, "output pointer is null");
    if (where == MDG_DEVICE) {
        CK(launch_positions_out(s, x), "positions out");
    } else {
        CK(launch_positions_out(s, s->fout), "positions out");
        CK(cudaMemcpyAsync(x, s->fout, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToHost,
                           s->stream),
           "copy");
    }
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return read_status(s);
}

MDG_API int mdg_get_velocities(mdg_system *s, double *v, int where) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!v) return fail(MDG_ERR_INVALID, "output pointer is null");
    CK(cudaMemcpyAsync(v, s->v, sizeof(double) * 3 * s->n,
                       where == MDG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       s->stream),
       "copy velocities");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return MDG_OK;
}

MDG_API int mdg_compute_forces(mdg_system *s, unsigned mask) {
    int rc = check_sys(s);
    if (rc) return rc;
    mask &= MDG_MASK_ALL;
    rc = ready_for_forces(s, mask);
    if (rc) return rc;
    rc = evaluate(s, mask, 1);
    if (rc) return rc;
    s->forces_valid = 1;
    s->forces_mask = mask;
    s->forces_weight = 1.0f;
    CK(cudaGetLastError(), "compute forces");
    return MDG_OK;
}

MDG_API int mdg_get_forces(mdg_system *s, double *f, int where) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!f) return fail(MDG_ERR_INVALID, "output pointer is null");
    if (!s->forces_valid) return fail(MDG_ERR_STATE, "no force evaluation since the last change");
    CK(launch_forces_out(s), "forces out");
    CK(cudaMemcpyAsync(f, s->fout, sizeof(double) * 3 * s->n,
                       where == MDG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       s->stream),
       "copy forces");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return read_status(s);
}

MDG_API int mdg_get_energies_batch(mdg_system *s, double *energies, double *kinetic) {
    int rc = check_sys(s);
    if (rc) return rc;
    std::vector<long long> e((size_t)kEnergySlots * s->n_sys);
    CK(cudaMemcpyAsync(e.data(), s->energy, sizeof(long long) * e.size(), cudaMemcpyDeviceToHost,
                       s->stream),
       "copy");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    rc = read_status(s);
    if (rc) return rc;
    const bool recip = (s->forces_mask & MDG_MASK(MDG_TERM_COUL_RECIP)) && s->pme.on;
    for (int q = 0; q < s->n_sys; ++q) {
        const long long *eq = e.data() + (size_t)kEnergySlots * q;
        if (energies) {
            double *out = energies + (size_t)MDG_NUM_TERMS * q;
            for (int t = 0; t < MDG_NUM_TERMS; ++t) out[t] = (double)eq[t] * kFixInv;
            if (recip) out[MDG_TERM_COUL_RECIP] += s->e_self[q] + s->e_net[q];
        }
        if (kinetic) kinetic[q] = (double)eq[kSlotKinetic] * kFixInv;
    }
    return MDG_OK;
}

namespace {
// energy words + status word of one snapshot slot
size_t snap_words(const mdg_system *s) { return (size_t)kEnergySlots * s->n_sys + 1; }

// energies[MDG_NUM_TERMS] (sums over the batch) and the kinetic energy from
// kEnergySlots * n_sys fixed-point words, as mdg_get_energies reports them
void energies_from_words(const mdg_system *s, const long long *e, bool recip, double *energies,
                         double *kinetic) {
    if (energies)
        for (int t = 0; t < MDG_NUM_TERMS; ++t) {
            double a = 0.0;
            for (int q = 0; q < s->n_sys; ++q) {
                a += (double)e[(size_t)kEnergySlots * q + t] * kFixInv;
                if (recip && t == MDG_TERM_COUL_RECIP) a += s->e_self[q] + s->e_net[q];
            }
            energies[t] = a;
        }
    if (kinetic) {
        double a = 0.0;
        for (int q = 0; q < s->n_sys; ++q) a += (double)e[(size_t)kEnergySlots * q + kSlotKinetic] * kFixInv;
        *kinetic = a;
    }
}
}  // namespace

MDG_API int mdg_energy_snapshot(mdg_system *s, int slot) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (slot < 0 || slot >= MDG_SNAPSHOT_SLOTS)
        return fail(MDG_ERR_INVALID, "snapshot slot %d outside [0, %d)", slot, MDG_SNAPSHOT_SLOTS);
    const size_t w = snap_words(s);
    if (!s->snap_host) {
        long long *h = nullptr;
        CK(cudaMallocHost((void **)&h, sizeof(long long) * w * MDG_SNAPSHOT_SLOTS),
           "pinned snapshot ring");
        s->snap_host = h;
    }
    if (!s->snap_ev[slot])
        CK(cudaEventCreateWithFlags(&s->snap_ev[slot], cudaEventDisableTiming), "event");
    long long *dst = s->snap_host + w * slot;
    CK(cudaMemcpyAsync(dst, s->energy, sizeof(long long) * (w - 1), cudaMemcpyDeviceToHost,
                       s->stream),
       "copy energies");
    // the status int lands in the low half of the last word (the read masks)
    CK(cudaMemcpyAsync(dst + w - 1, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream),
       "status read");
    CK(cudaEventRecord(s->snap_ev[slot], s->stream), "event record");
    s->snap_mask[slot] = s->forces_mask;
    s->snap_recip[slot] = (s->forces_mask & MDG_MASK(MDG_TERM_COUL_RECIP)) && s->pme.on;
    s->snap_taken[slot] = true;
    return MDG_OK;
}

MDG_API int mdg_energy_snapshot_read(mdg_system *s, int slot, int wait, double *energies,
                                     double *kinetic, int *ready) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (slot < 0 || slot >= MDG_SNAPSHOT_SLOTS)
        return fail(MDG_ERR_INVALID, "snapshot slot %d outside [0, %d)", slot, MDG_SNAPSHOT_SLOTS);
    if (!s->snap_taken[slot]) return fail(MDG_ERR_STATE, "snapshot slot %d holds no snapshot", slot);
    if (!wait && !ready) return fail(MDG_ERR_INVALID, "a non-waiting read needs `ready`");
    if (wait) {
        CK(cudaEventSynchronize(s->snap_ev[slot]), "synchronize");
    } else {
        const cudaError_t q = cudaEventQuery(s->snap_ev[slot]);
        if (q == cudaErrorNotReady) {
            *ready = 0;
            return MDG_OK;
        }
        CK(q, "event query");
    }
    if (ready) *ready = 1;
    const size_t w = snap_words(s);
    const long long *src = s->snap_host + w * slot;
    const int st = (int)(src[w - 1] & 0xffffffffll);
    if (st) return decode_status(s, st);
    energies_from_words(s, src, s->snap_recip[slot], energies, kinetic);
    return MDG_OK;
}

MDG_API int mdg_get_energies(mdg_system *s, double *energies, double *kinetic) {
    int rc = check_sys(s);
    if (rc) return rc;
    std::vector<double> e((size_t)MDG_NUM_TERMS * s->n_sys), k(s->n_sys);
    rc = mdg_get_energies_batch(s, e.data(), k.data());
    if (rc) return rc;
    if (energies)
        for (int t = 0; t < MDG_NUM_TERMS; ++t) {
            double a = 0.0;
            for (int q = 0; q < s->n_sys; ++q) a += e[(size_t)MDG_NUM_TERMS * q + t];
            energies[t] = a;
        }
    if (kinetic) {
        double a = 0.0;
        for (int q = 0; q < s->n_sys; ++q) a += k[q];
        *kinetic = a;
    }
    return MDG_OK;
}

MDG_API int mdg_kinetic_energy(mdg_system *s, double *kinetic) {
    int rc = check_sys(s);
    if (rc) return rc;
    CK(cudaMemset2DAsync(s->energy + kSlotKinetic, sizeof(long long) * kEnergySlots, 0,
                         sizeof(long long), s->n_sys, s->stream),
       "memset");
    CK(launch_kinetic(s), "kinetic");
    std::vector<long long> e((size_t)kEnergySlots * s->n_sys);
    CK(cudaMemcpyAsync(e.data(), s->energy, sizeof(long long) * e.size(), cudaMemcpyDeviceToHost,
                       s->stream),
       "copy");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    double a = 0.0;
    for (int q = 0; q < s->n_sys; ++q) a += (double)e[(size_t)kEnergySlots * q + kSlotKinetic] * kFixInv;
    if (kinetic) *kinetic = a;
    return MDG_OK;
}

MDG_API int mdg_kinetic_energies_noalloc(mdg_system *s, double *kinetic) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!kinetic) return fail(MDG_ERR_INVALID, "kinetic is null");
    if (s->n_sys > MDG_NOALLOC_MAX_SYSTEMS)
        return fail(MDG_ERR_INVALID,
                    "%d systems exceed the no-allocation scratch (at most %d systems)", s->n_sys,
                    MDG_NOALLOC_MAX_SYSTEMS);
    long long *acc = nullptr;
    CK(noalloc_scratch(s->device, &acc), "cudaGetSymbolAddress of the scratch array");
    // the accumulators start at zero
    CK(cudaMemsetAsync(acc, 0, sizeof(long long) * kEnergySlots * s->n_sys, s->stream),
       "memset");
    CK(launch_kinetic_scratch(s, acc), "kinetic");
    s->launches += 1;
    // each system's int64 kinetic word, into the caller's array, converted in place
    CK(cudaMemcpy2DAsync(kinetic, sizeof(double), acc + kSlotKinetic,
                         sizeof(long long) * kEnergySlots, sizeof(long long), s->n_sys,
                         cudaMemcpyDeviceToHost, s->stream),
       "copy");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    for (int q = 0; q < s->n_sys; ++q) {
        long long v;
        std::memcpy(&v, &kinetic[q], sizeof(v));
        kinetic[q] = (double)v * kFixInv;
    }
    return MDG_OK;
}

static int apply_shape(mdg_system *s, const int *sh) {
    const int split = sh[MDG_SHAPE_SPLIT], persistent = sh[MDG_SHAPE_PERSISTENT],
              pme_block = sh[MDG_SHAPE_PME_BLOCK], side_priority = sh[MDG_SHAPE_SIDE_PRIORITY],
              split_rings = sh[MDG_SHAPE_SPLIT_RINGS], pme_tiles = sh[MDG_SHAPE_PME_TILES],
              half = sh[MDG_SHAPE_HALF];
    if (split != 1 && split != 2 && split != 4 && split != 8 && split != 16)
        return fail(MDG_ERR_INVALID, "split %d is not 1, 2, 4, 8 or 16", split);
    if (persistent < 0 || persistent > 24)
        return fail(MDG_ERR_INVALID, "persistent CTAs per SM %d not in 0..24", persistent);
    if (pme_block != 64 && pme_block != 128 && pme_block != 256)
        return fail(MDG_ERR_INVALID, "PME block %d is not 64, 128 or 256", pme_block);
    if (side_priority != 0 && side_priority != 1)
        return fail(MDG_ERR_INVALID, "side priority must be 0 or 1");
    if (split_rings != 0 && split_rings != 1)
        return fail(MDG_ERR_INVALID, "split_rings must be 0 or 1");
    if (pme_tiles < 0 || pme_tiles > 3)
        return fail(MDG_ERR_INVALID, "pme_tiles %d not in 0..3", pme_tiles);
    if (half < 0 || half > 2) return fail(MDG_ERR_INVALID, "half must be 0, 1 or 2");
    s->nb_split = split;
    s->nb_persistent = persistent;
    s->nb_persistent_ctas = persistent * s->n_sms;
    s->pme_block = pme_block;
    s->side_priority = side_priority;
    s->side_stream = s->side_streams[side_priority];
    s->bond_stream = s->bond_streams[side_priority];
    s->nb_split_rings = split_rings;
    s->pme_tiles = pme_tiles;
    s->nb_half = half;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

static void current_shape(const mdg_system *s, int *sh) {
    sh[MDG_SHAPE_SPLIT] = s->nb_split;
    sh[MDG_SHAPE_PERSISTENT] = s->nb_persistent;
    sh[MDG_SHAPE_PME_BLOCK] = s->pme_block;
    sh[MDG_SHAPE_SIDE_PRIORITY] = s->side_priority;
    sh[MDG_SHAPE_SPLIT_RINGS] = s->nb_split_rings;
    sh[MDG_SHAPE_PME_TILES] = s->pme_tiles;
    sh[MDG_SHAPE_HALF] = s->nb_half;
}

MDG_API int mdg_set_launch_shape(mdg_system *s, const int *shape) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!shape) return fail(MDG_ERR_INVALID, "shape is null");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    CK(cudaStreamSynchronize(s->side_stream), "synchronize");
    CK(cudaStreamSynchronize(s->bond_stream), "synchronize");
    return apply_shape(s, shape);
}

MDG_API int mdg_get_launch_shape(mdg_system *s, int *shape) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!shape) return fail(MDG_ERR_INVALID, "shape is null");
    current_shape(s, shape);
    return MDG_OK;
}

// The autotuner.  With an integrator configured it times MD steps exactly
// as mdg_integrate runs them (one captured single-step graph per shape,
// replayed from the saved state, each replay between its own pair of events
// so host launch gaps do not count), and puts the state back afterwards;
// otherwise it times force evaluations of `mask`.  Phase one varies the pair
// kernel (work items per cluster 2/4/8 x one CTA per item or 20/24 resident
// CTAs per SM x split rings x i groups of 32 / 16 / 8 atoms) with the PME fields of the shape
// in use; phase
// two varies PME and the streams (block 64/128/256 x tiles 0-3 x side
// priority) with phase one's best pair kernel; phase three re-times the four
// fastest and the shape in use, interleaved, 4 x reps each, and keeps the
// fastest (shapes a percent apart are otherwise decided by noise).
MDG_API int mdg_autotune(mdg_system *s, unsigned mask, int reps, double *best_ms) {
    int rc = check_sys(s);
    if (rc) return rc;
    mask &= MDG_MASK_ALL;
    rc = ready_for_forces(s, mask);
    if (rc) return rc;
    if (reps < 1 || reps > 1000) return fail(MDG_ERR_INVALID, "reps %d out of range", reps);
    const bool steps = s->integ_kind >= 0 && s->have_masses;
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    rc = evaluate(s, mask, 0);  // re-sorted clusters, fresh boxes, valid forces
    if (rc) return rc;
    double *xs = nullptr, *vs = nullptr;
    unsigned long long step_saved = 0;
    if (steps) {
        if ((rc = dalloc(&xs, 3 * (size_t)s->n)) || (rc = dalloc(&vs, 3 * (size_t)s->n))) {
            dfree(xs);
            return rc;
        }
        cudaMemcpyAsync(xs, s->x, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(vs, s->v, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(&step_saved, s->step_dev, sizeof(step_saved), cudaMemcpyDeviceToHost,
                        s->stream);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    struct Shape {
        int sh[MDG_SHAPE_FIELDS];
        float ms;
    };
    auto time_shape = [&](Shape &c, int n) -> int {
        int r = apply_shape(s, c.sh);
        Graph g;
        if (!r && steps) {
            cudaMemcpyAsync(s->x, xs, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice,
                            s->stream);
            cudaMemcpyAsync(s->v, vs, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice,
                            s->stream);
            r = evaluate(s, mask, 0);  // forces of the restored positions
            if (!r) r = capture_steps(s, g, 1, 0, mask);
        }
        float total = 0.f;
        for (int w = 0; w < 2 + n && !r && ce == cudaSuccess; ++w) {
            ce = cudaEventRecord(e0, s->stream);
            if (ce != cudaSuccess) break;
            if (steps) ce = cudaGraphLaunch(g.exec, s->stream);
            else r = evaluate(s, mask, 0);
            if (r || ce != cudaSuccess) break;
            ce = cudaEventRecord(e1, s->stream);
            if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
            if (w >= 2) total += ms;
        }
        if (g.exec) cudaGraphExecDestroy(g.exec);
        c.ms = total / n;
        return r;
    };
    auto by_time = [](const Shape &x, const Shape &y) { return x.ms < y.ms; };
    Shape current;
    current_shape(s, current.sh);
    current.ms = 0.f;
    const bool pme = (mask & MDG_MASK(MDG_TERM_COUL_RECIP)) && s->pme.on;
    std::vector<Shape> tried;
    // phase one: the pair kernel
    for (int sp : {2, 4, 8})
        for (int pe : {0, 20, 24})
            for (int sr = 0; sr <= 1; ++sr)
                for (int hf = 0; hf <= 2 && !rc && ce == cudaSuccess; ++hf) {
                    Shape c = current;
                    c.sh[MDG_SHAPE_SPLIT] = sp;
                    c.sh[MDG_SHAPE_PERSISTENT] = pe;
                    c.sh[MDG_SHAPE_SPLIT_RINGS] = sr;
                    c.sh[MDG_SHAPE_HALF] = hf;
                    rc = time_shape(c, reps);
                    tried.push_back(c);
                }
    // phase two: PME and the side streams
    if (!rc && ce == cudaSuccess) {
        const Shape base = *std::min_element(tried.begin(), tried.end(), by_time);
        for (int bl : {64, 128, 256})
            for (int tl = 0; tl < 4; ++tl)
                for (int pr = 0; pr <= 1 && !rc && ce == cudaSuccess; ++pr) {
                    if (!pme && (bl != 256 || tl != 0)) continue;
                    Shape c = base;
                    c.sh[MDG_SHAPE_PME_BLOCK] = bl;
                    c.sh[MDG_SHAPE_PME_TILES] = tl;
                    c.sh[MDG_SHAPE_SIDE_PRIORITY] = pr;
                    rc = time_shape(c, reps);
                    tried.push_back(c);
                }
    }
    Shape best = current;
    float best_t = 0.f;
    if (!rc && ce == cudaSuccess) {
        std::sort(tried.begin(), tried.end(), by_time);
        std::vector<Shape> top(tried.begin(), tried.begin() + std::min<size_t>(4, tried.size()));
        top.push_back(current);
        std::vector<float> sum(top.size(), 0.f);
        for (int round = 0; round < 4 && !rc && ce == cudaSuccess; ++round)
            for (size_t k = 0; k < top.size() && !rc && ce == cudaSuccess; ++k) {
                rc = time_shape(top[k], reps);
                sum[k] += top[k].ms;
            }
        size_t b = 0;
        for (size_t k = 1; k < top.size(); ++k)
            if (sum[k] < sum[b]) b = k;
        best = top[b];
        best_t = sum[b] / 4.0f;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    const int ra = apply_shape(s, best.sh);
    if (steps) {
        // put the state back: positions, velocities, the noise counter
        cudaMemcpyAsync(s->x, xs, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->v, vs, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->step_dev, &step_saved, sizeof(step_saved), cudaMemcpyHostToDevice,
                        s->stream);
        cudaStreamSynchronize(s->stream);
        dfree(xs);
        dfree(vs);
        s->need_reorder = 1;
    }
    s->forces_valid = 0;
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "autotune");
    if (ra) return ra;
    rc = read_status(s);
    if (rc) return rc;
    if (best_ms) *best_ms = best_t;
    return MDG_OK;
}

MDG_API int mdg_minimize_step(mdg_system *s, double alpha) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!(alpha > 0) || !std::isfinite(alpha))
        return fail(MDG_ERR_INVALID, "step length %g must be positive", alpha);
    if (!s->forces_valid) return fail(MDG_ERR_STATE, "no force evaluation since the last change");
    CK(launch_sd_step(s, alpha), "steepest-descent step");
    s->forces_valid = 0;
    if (++s->steps_since_reorder >= s->reorder_interval) s->need_reorder = 1;
    return MDG_OK;
}

MDG_API int mdg_step_host(mdg_system *s, const double *x_in, const double *v_in, int n_steps,
                          unsigned mask, double *x_out, double *v_out, double *energies,
                          double *kinetic) {
    int rc = check_sys(s);
    if (rc) return rc;
    const size_t ne = (size_t)kEnergySlots * s->n_sys;
    if (!s->host_stage || !s->xin || !s->same_flag) {
        // pinned staging for the energy words, the status word and the
        // positions-comparison flag; each buffer is allocated once, so a
        // failed call leaves nothing half set up for the next one
        if (!s->host_stage)
            CK(cudaMallocHost((void **)&s->host_stage, sizeof(long long) * (ne + 2)),
               "pinned staging");
        int rc2 = s->xin ? 0 : dalloc(&s->xin, 3 * (size_t)s->n);
        if (!rc2 && !s->same_flag) rc2 = dalloc(&s->same_flag, 1);
        if (rc2) return fail(rc2, "step_host staging");
    }
    long long *stage = s->host_stage;
    // Positions that equal the state (as the previous call returned it) keep
    // the forces already computed for them and the cluster order.  The copy
    // lands beside the state and a comparison kernel flags any difference;
    // the steps run on the device state meanwhile (speculatively), and the
    // flag comes back with the results.  If the positions differed, the
    // state before the call is put back and the call is redone from the
    // incoming positions (re-sort, fresh force evaluation).  A learned slow
    // force keeps more state than positions and velocities: there the flag
    // is read before the steps.
    bool speculate = false;
    const uint64_t step0 = s->step;
    const int since0 = s->steps_since_reorder;
    if (x_in) {
        CK(cudaMemcpyAsync(s->xin, x_in, sizeof(double) * 3 * s->n, cudaMemcpyHostToDevice,
                           s->stream),
           "copy positions");
        bool same = false;
        if (s->have_x && s->forces_valid) {
            CK(cudaMemsetAsync(s->same_flag, 0, sizeof(int), s->stream), "memset");
            CK(launch_same_positions(s, s->xin, s->same_flag), "compare positions");
            if (!ls_active(s)) {
                if (!v_in) {  // the velocities to restore should the step be redone
                    if (!s->vsave && (rc = dalloc(&s->vsave, 3 * (size_t)s->n)))
                        return fail(rc, "step_host staging");
                    CK(cudaMemcpyAsync(s->vsave, s->v, sizeof(double) * 3 * s->n,
                                       cudaMemcpyDeviceToDevice, s->stream),
                       "save velocities");
                }
                speculate = true;
                same = true;
            } else {
                CK(cudaMemcpyAsync(stage + ne + 1, s->same_flag, sizeof(int),
                                   cudaMemcpyDeviceToHost, s->stream),
                   "flag read");
                CK(cudaStreamSynchronize(s->stream), "synchronize");
                same = ((int)(stage[ne + 1] & 0xffffffffll)) == 0;
            }
        }
        if (!same) {
            CK(cudaMemcpyAsync(s->x, s->xin, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToDevice,
                               s->stream),
               "copy positions");
            s->have_x = 1;
            s->need_reorder = 1;
            s->forces_valid = 0;
        }
    }
    if (v_in) {
        CK(cudaMemcpyAsync(s->v, v_in, sizeof(double) * 3 * s->n, cudaMemcpyHostToDevice,
                           s->stream),
           "copy velocities");
        s->have_v = 1;
    }
    const int want_energy = (energies || kinetic) ? 1 : 0;
    rc = mdg_integrate(s, n_steps, mask, want_energy);
    if (rc) {
        cudaStreamSynchronize(s->stream);
        return rc;
    }
    if (x_out) {
        CK(launch_positions_out(s, s->fout), "positions out");
        CK(cudaMemcpyAsync(x_out, s->fout, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToHost,
                           s->stream),
           "copy positions");
    }
    if (v_out)
        CK(cudaMemcpyAsync(v_out, s->v, sizeof(double) * 3 * s->n, cudaMemcpyDeviceToHost,
                           s->stream),
           "copy velocities");
    if (want_energy)
        CK(cudaMemcpyAsync(stage, s->energy, sizeof(long long) * ne, cudaMemcpyDeviceToHost,
                           s->stream),
           "copy energies");
    CK(cudaMemcpyAsync(stage + ne, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream),
       "status read");
    if (speculate)
        CK(cudaMemcpyAsync(stage + ne + 1, s->same_flag, sizeof(int), cudaMemcpyDeviceToHost,
                           s->stream),
           "flag read");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    if (speculate && (int)(stage[ne + 1] & 0xffffffffll) != 0) {
        // the positions differed: the speculative steps and anything they
        // raised are void; back to the state before the call, then redo
        // from the incoming positions
        CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
        if (!v_in)
            CK(cudaMemcpyAsync(s->v, s->vsave, sizeof(double) * 3 * s->n,
                               cudaMemcpyDeviceToDevice, s->stream),
               "restore velocities");
        // the step counter lives on the device too (the captured steps
        // advance it there): both go back
        if ((rc = mdg_set_step(s, step0))) return rc;
        s->steps_since_reorder = since0;
        s->forces_valid = 0;  // the redo takes the incoming positions as new
        return mdg_step_host(s, x_in, v_in, n_steps, mask, x_out, v_out, energies, kinetic);
    }
    const int st = (int)(stage[ne] & 0xffffffffll);
    if (st) {
        CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
        CK(cudaStreamSynchronize(s->stream), "synchronize");
        return decode_status(s, st);
    }
    const bool recip = (s->forces_mask & MDG_MASK(MDG_TERM_COUL_RECIP)) && s->pme.on;
    if (energies)
        for (int t = 0; t < MDG_NUM_TERMS; ++t) {
            double a = 0.0;
            for (int q = 0; q < s->n_sys; ++q) {
                a += (double)stage[(size_t)kEnergySlots * q + t] * kFixInv;
                if (t == MDG_TERM_COUL_RECIP && recip) a += s->e_self[q] + s->e_net[q];
            }
            energies[t] = a;
        }
    if (kinetic) {
        double a = 0.0;
        for (int q = 0; q < s->n_sys; ++q)
            a += (double)stage[(size_t)kEnergySlots * q + kSlotKinetic] * kFixInv;
        *kinetic = a;
    }
    return MDG_OK;
}

MDG_API int mdg_set_mts(mdg_system *s, int k) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (k < 1 || k > 16) return fail(MDG_ERR_INVALID, "outer step %d not in 1..16", k);
    s->mts_k = k;
    if (s->ls) s->ls->enabled = 0;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

// ---- learned slow force ------------------------------------------------------

MDG_API int mdg_learned_config(mdg_system *s, double rf, double skin, int list_capacity) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (s->n_sys != 1) return fail(MDG_ERR_INVALID, "the learned slow force takes one system");
    if (!(rf >= 2.0 && rf <= 12.0)) return fail(MDG_ERR_INVALID, "rf %g not in [2, 12] A", rf);
    if (!(skin >= 0.0 && skin <= 4.0)) return fail(MDG_ERR_INVALID, "skin %g not in [0, 4] A", skin);
    if (list_capacity < 16 || list_capacity > 4096)
        return fail(MDG_ERR_INVALID, "list capacity %d not in 16..4096", list_capacity);
    for (int k = 0; k < 3; ++k)
        if (s->sys_h[0].Ld[k] < 3.0 * (rf + skin))
            return fail(MDG_ERR_INVALID, "box edge %g A below 3 (rf + skin)", s->sys_h[0].Ld[k]);
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    const int was_on = s->ls ? s->ls->enabled : 0, k = s->ls ? s->ls->k : 4;
    const float thr = s->ls ? s->ls->threshold : 1e-3f;
    const int tc = s->ls ? s->ls->use_tc : 1;
    const int ty = s->ls ? s->ls->use_taylor : 0, nt = s->ls ? s->ls->use_net : 1;
    rc = ls_configure(s, (float)rf, (float)skin, list_capacity);
    if (rc) return fail(rc, "learned slow force: allocation failed");
    s->ls->use_taylor = ty;
    s->ls->use_net = nt;
    s->ls->enabled = was_on;
    s->ls->k = k;
    s->ls->threshold = thr;
    s->ls->use_tc = tc;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

static int ls_check(mdg_system *s) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!s->ls) return fail(MDG_ERR_STATE, "learned slow force not configured");
    return MDG_OK;
}

MDG_API int mdg_learned_num_params(int32_t *n) {
    if (!n) return fail(MDG_ERR_INVALID, "null argument");
    *n = kLsParams;
    return MDG_OK;
}

MDG_API int mdg_learned_set_params(mdg_system *s, const float *params, int32_t n) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (!params || n != kLsParams) return fail(MDG_ERR_INVALID, "expected %d parameters", kLsParams);
    for (int k = 0; k < n; ++k)
        if (!std::isfinite(params[k])) return fail(MDG_ERR_INVALID, "parameter %d not finite", k);
    CK(cudaMemcpyAsync(s->ls->params, params, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream),
       "copy");
    CK(cudaMemsetAsync(s->ls->adam_m, 0, sizeof(float) * kLsParams, s->stream), "memset");
    CK(cudaMemsetAsync(s->ls->adam_v, 0, sizeof(float) * kLsParams, s->stream), "memset");
    CK(ls_refresh_weights(s), "weights");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    s->ls->trained = 1;
    s->forces_valid = 0;
    return MDG_OK;
}

MDG_API int mdg_learned_get_params(mdg_system *s, float *params, int32_t n) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (!params || n != kLsParams) return fail(MDG_ERR_INVALID, "expected %d parameters", kLsParams);
    CK(cudaMemcpyAsync(params, s->ls->params, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream),
       "copy");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return MDG_OK;
}

MDG_API int mdg_learned_frame(mdg_system *s, int32_t slot) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (slot != 0 && slot != 1) return fail(MDG_ERR_INVALID, "slot %d not 0 or 1", slot);
    const unsigned mask = MDG_MASK(MDG_TERM_COUL_RECIP);
    rc = ready_for_forces(s, mask);
    if (rc) return rc;
    if (!s->pme.on) return fail(MDG_ERR_STATE, "PME has not been configured");
    s->ls_slot = slot;
    s->ls_phase = kLsFrame;
    s->slow_target = s->ls->fs;
    s->recip_weight = 1.0f;
    rc = evaluate(s, mask, 0);
    s->ls_phase = kLsOff;
    s->slow_target = nullptr;
    s->forces_valid = 0;  // f now holds no complete force
    if (rc) return rc;
    return read_status(s);
}

MDG_API int mdg_learned_frame_data(mdg_system *s, int32_t slot, float *features, float *vectors,
                                   float *slow_force, float *predicted) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (slot != 0 && slot != 1) return fail(MDG_ERR_INVALID, "slot %d not 0 or 1", slot);
    const Learned &L = *s->ls;
    const size_t n = s->n;
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    if (features)
        CK(cudaMemcpy(features, L.xraw[slot], sizeof(float) * n * kLsFeat, cudaMemcpyDeviceToHost),
           "copy");
    if (vectors || slow_force || predicted) {
        std::vector<float> buf;
        if (vectors)
            CK(cudaMemcpy(vectors, L.S[slot], sizeof(float) * 3 * kLsVec * n, cudaMemcpyDeviceToHost),
               "copy");
        if (slow_force) {
            buf.resize(3 * n);
            CK(cudaMemcpy(buf.data(), L.T[slot], sizeof(float) * 3 * n, cudaMemcpyDeviceToHost), "copy");
            for (size_t i = 0; i < n; ++i)
                for (int d = 0; d < 3; ++d) slow_force[3 * i + d] = buf[(size_t)d * n + i];
        }
        if (predicted) {
            buf.resize((size_t)3 * L.n_rows);
            CK(cudaMemcpy(buf.data(), L.G[slot], sizeof(float) * buf.size(), cudaMemcpyDeviceToHost),
               "copy");
            for (size_t i = 0; i < n; ++i)
                for (int d = 0; d < 3; ++d) predicted[3 * i + d] = buf[(size_t)d * L.n_rows + i];
        }
    }
    return MDG_OK;
}

MDG_API int mdg_learned_predict(mdg_system *s, int32_t slot, float *predicted) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (slot != 0 && slot != 1) return fail(MDG_ERR_INVALID, "slot %d not 0 or 1", slot);
    CK(ls_predict(s, slot), "learned prediction");
    rc = read_status(s);
    if (rc) return rc;
    return predicted ? mdg_learned_frame_data(s, slot, nullptr, nullptr, nullptr, predicted)
                     : MDG_OK;
}

MDG_API int mdg_learned_train_step(mdg_system *s, float lr, int32_t t, double *loss) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (!(lr > 0.f) || t < 1) return fail(MDG_ERR_INVALID, "lr must be > 0 and t >= 1");
    CK(ls_train(s, lr, t, loss), "train step");
    s->ls->trained = 1;
    return read_status(s);
}

MDG_API int mdg_set_mts_learned(mdg_system *s, int32_t k, double threshold) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (k == 0 || k == 1) {
        if (s->ls) s->ls->enabled = 0;
        s->mts_k = 1;
    } else {
        rc = ls_check(s);
        if (rc) return rc;
        if (k < 2 || k > 16) return fail(MDG_ERR_INVALID, "outer step %d not in 2..16", k);
        if (!(threshold > 0.0)) return fail(MDG_ERR_INVALID, "threshold must be positive");
        if (!s->pme.on) return fail(MDG_ERR_STATE, "PME has not been configured");
        s->ls->enabled = 1;
        s->ls->k = k;
        s->ls->threshold = (float)threshold;
        s->mts_k = k;
        CK(cudaMemsetAsync(s->ls->mode, 0, sizeof(int) * 2, s->stream), "memset");
    }
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_learned_set_kernel(mdg_system *s, int32_t tensor_cores) {
    int rc = ls_check(s);
    if (rc) return rc;
    s->ls->use_tc = tensor_cores ? 1 : 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_learned_wait_test(mdg_system *s) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (!s->ls->use_tc) return fail(MDG_ERR_STATE, "the tensor-core kernel is not selected");
    s->ls->tc_wait_test = 1;
    drop_graph(s);  // the next launch must be an eager one
    return MDG_OK;
}

MDG_API int mdg_learned_set_terms(mdg_system *s, int32_t field_gradient, int32_t network) {
    int rc = ls_check(s);
    if (rc) return rc;
    s->ls->use_taylor = field_gradient ? 1 : 0;
    s->ls->use_net = network ? 1 : 0;
    s->forces_valid = 0;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_learned_stats(mdg_system *s, double *out8) {
    int rc = ls_check(s);
    if (rc) return rc;
    if (!out8) return fail(MDG_ERR_INVALID, "null argument");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    CK(cudaMemcpy(out8, s->ls->stats, sizeof(double) * 8, cudaMemcpyDeviceToHost), "copy");
    int mode[2] = {0, 0};
    CK(cudaMemcpy(mode, s->ls->mode, sizeof(mode), cudaMemcpyDeviceToHost), "copy");
    out8[7] = mode[0];
    return MDG_OK;
}

MDG_API int mdg_learned_reset_stats(mdg_system *s) {
    int rc = ls_check(s);
    if (rc) return rc;
    CK(cudaMemsetAsync(s->ls->stats, 0, sizeof(double) * 5, s->stream), "memset");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return MDG_OK;
}

MDG_API int mdg_integrator_config(mdg_system *s, int kind, double dt, double temperature,
                                  double friction, uint64_t seed) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (kind != MDG_INTEGRATOR_VERLET && kind != MDG_INTEGRATOR_LANGEVIN)
        return fail(MDG_ERR_INVALID, "unknown integrator %d", kind);
    if (!(dt > 0)) return fail(MDG_ERR_INVALID, "time step must be positive");
    if (kind == MDG_INTEGRATOR_LANGEVIN && (!(temperature >= 0) || !(friction >= 0)))
        return fail(MDG_ERR_INVALID, "temperature and friction must be >= 0");
    s->integ_kind = kind;
    s->dt = dt;
    s->temperature = temperature;
    s->friction = kind == MDG_INTEGRATOR_LANGEVIN ? friction : 0.0;
    s->seed = seed;
    drop_graph(s);
    return MDG_OK;
}

MDG_API int mdg_get_step(mdg_system *s, uint64_t *step) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (step) *step = s->step;
    return MDG_OK;
}

MDG_API int mdg_set_step(mdg_system *s, uint64_t step) {
    int rc = check_sys(s);
    if (rc) return rc;
    unsigned long long v = step;
    CK(cudaMemcpyAsync(s->step_dev, &v, sizeof(v), cudaMemcpyHostToDevice, s->stream), "copy");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    s->step = step;
    return MDG_OK;
}

MDG_API int mdg_integrate(mdg_system *s, int n_steps, unsigned mask, int want_energy) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (n_steps < 0) return fail(MDG_ERR_INVALID, "negative step count");
    if (s->integ_kind < 0) return fail(MDG_ERR_STATE, "integrator has not been configured");
    mask &= MDG_MASK_ALL;
    rc = ready_for_forces(s, mask);
    if (rc) return rc;
    if (!s->have_masses) return fail(MDG_ERR_STATE, "masses have not been set");
    if (s->graph.exec && s->graph.mask != mask) drop_graph(s);
    for (auto &plane : s->graph_step)
        for (auto &row : plane)
            for (Graph &g : row)
                if (g.exec && g.mask != mask) drop_graph(s);
    for (Graph &g : s->graph_eval)
        if (g.exec && g.mask != mask) drop_graph(s);
    // the force buffer the first pre-force update uses: multiple time steps
    // want the weight of the evaluation that ended the previous step
    const float want_w = ls_active(s) ? -1.0f
                         : s->step == 0 ? mts_weight(s, (uint64_t)s->mts_k - 1)
                                        : mts_weight(s, s->step - 1);
    if (!s->forces_valid || s->forces_mask != mask || s->forces_weight != want_w) {
        if (ls_active(s)) {
            // learned form: a full evaluation anchors the prediction
            rc = ls_evaluate(s, mask, 0, kLsAnchor);
            if (rc) return rc;
        } else if (s->mts_k > 1) {
            s->recip_weight = want_w;
            rc = evaluate(s, mask, 0);
            s->recip_weight = 1.0f;
            if (rc) return rc;
            s->forces_weight = want_w;
        } else if (s->graph_mode == MDG_GRAPH_STEP && n_steps > 0) {
            const int resort = s->need_reorder ? 1 : 0;
            Graph &g = s->graph_eval[resort];
            if (!g.exec) {
                rc = capture_eval(s, g, resort, mask);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(g.exec, s->stream), "graph launch");
            s->launches += g.steps;
            if (resort) {
                s->need_reorder = 0;
                s->steps_since_reorder = 0;
            }
        } else {
            rc = evaluate(s, mask, 1);
            if (rc) return rc;
        }
        s->forces_valid = 1;
        s->forces_mask = mask;
    }
    const int R = s->reorder_interval;
    int remaining = n_steps;
    while (remaining > 0) {
        const bool chunk_start = s->need_reorder || s->steps_since_reorder >= R;
        const int usable = remaining - (want_energy ? 1 : 0);
        if (s->graph_mode == MDG_GRAPH_STEP || s->mts_k > 1) {
            const int e = (want_energy && remaining == 1) ? 1 : 0;
            const int outer = mts_weight(s, s->step) != 0.f ? 1 : 0;
            Graph &g = s->graph_step[chunk_start ? 1 : 0][e][outer];
            if (!g.exec) {
                rc = capture_steps(s, g, 1, chunk_start, mask, e);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(g.exec, s->stream), "graph launch");
            s->launches += g.steps;
            s->need_reorder = 0;
            s->steps_since_reorder = chunk_start ? 1 : s->steps_since_reorder + 1;
            s->forces_weight = ls_active(s) ? -1.0f : mts_weight(s, s->step);
            s->step += 1;
            remaining -= 1;
        } else if (chunk_start && usable >= R && R >= 2) {
            if (!s->graph.exec) {
                rc = capture_steps(s, s->graph, R, 1, mask);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(s->graph.exec, s->stream), "graph launch");
            s->launches += s->graph.steps;
            s->need_reorder = 0;
            s->steps_since_reorder = R;
            s->step += R;
            remaining -= R;
        } else {
            const int e = (want_energy && remaining == 1) ? 1 : 0;
            rc = md_step(s, mask, e);
            if (rc) return rc;
            remaining -= 1;
        }
    }
    if (want_energy && n_steps == 0) {
        rc = evaluate(s, mask, 1);
        if (rc) return rc;
        s->forces_weight = 1.0f;
    }
    s->forces_valid = 1;
    s->forces_mask = mask;
    CK(cudaGetLastError(), "integrate");
    return MDG_OK;
}

MDG_API int mdg_pairset_dump(mdg_system *s, int32_t *pairs, int64_t capacity, int64_t *count) {
    int rc = check_sys(s);
    if (rc) return rc;
    rc = ready_for_forces(s, MDG_MASK(MDG_TERM_LJ) | MDG_MASK(MDG_TERM_COUL_REAL));
    if (rc) return rc;
    if (capacity < 0) return fail(MDG_ERR_INVALID, "negative capacity");
    if (s->need_reorder) {
        CK(launch_reorder(s), "reorder");
        s->need_reorder = 0;
        s->steps_since_reorder = 0;
    }
    CK(launch_pack(s), "pack");
    s->forces_valid = 0;  // pack zeroed the force slots
    int *buf = nullptr;
    if ((rc = dalloc(&buf, 2 * (size_t)std::max<int64_t>(capacity, 1)))) return rc;
    s->dump_buf = buf;
    s->dump_cap = capacity;
    CK(cudaMemsetAsync(s->dump_count, 0, sizeof(unsigned long long), s->stream), "memset");
    // the tile kernel covers LJ and Ewald real space; the pair set is the same
    const int saved_mode = s->coul_mode, saved_lj = s->lj_on;
    if (s->coul_mode == MDG_COUL_BARE) s->coul_mode = MDG_COUL_NONE;
    s->lj_on = 1;
    cudaError_t e = launch_nonbonded(s, MDG_MASK(MDG_TERM_LJ), 0, 1);
    if (e == cudaSuccess) e = launch_special(s, MDG_MASK(MDG_TERM_LJ), 0, 1);
    s->coul_mode = saved_mode;
    s->lj_on = saved_lj;
    unsigned long long got = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&got, s->dump_count, sizeof(got), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && pairs && capacity > 0)
        e = cudaMemcpy(pairs, buf, sizeof(int) * 2 * std::min<int64_t>(capacity, (int64_t)got),
                       cudaMemcpyDeviceToHost);
    cudaFree(buf);
    s->dump_buf = nullptr;
    s->dump_cap = 0;
    if (e != cudaSuccess) return cuda_fail(e, "pair dump");
    if (count) *count = (int64_t)got;
    if ((int64_t)got > capacity) return fail(MDG_ERR_CAPACITY, "%lld pairs exceed capacity %lld",
                                             (long long)got, (long long)capacity);
    return MDG_OK;
}

MDG_API int mdg_langevin_noise(mdg_system *s, uint64_t step, float *out) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!out) return fail(MDG_ERR_INVALID, "output pointer is null");
    float *d = nullptr;
    if ((rc = dalloc(&d, 3 * (size_t)s->n))) return rc;
    cudaError_t e = launch_noise(s, step, d);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d, sizeof(float) * 3 * s->n, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "noise");
    return MDG_OK;
}

MDG_API int mdg_check_status(mdg_system *s) {
    int rc = check_sys(s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return read_status(s);
}

MDG_API int mdg_nonbonded_stats(mdg_system *s, int64_t *stats) {
    int rc = check_sys(s);
    if (rc) return rc;
    unsigned long long v[4];
    CK(cudaMemcpyAsync(v, s->stats, sizeof(v), cudaMemcpyDeviceToHost, s->stream), "copy");
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    for (int k = 0; k < 4; ++k) stats[k] = (int64_t)v[k];
    return MDG_OK;
}

MDG_API int mdg_set_graph_mode(mdg_system *s, int mode) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (mode != MDG_GRAPH_CHUNK && mode != MDG_GRAPH_STEP)
        return fail(MDG_ERR_INVALID, "unknown graph mode %d", mode);
    s->graph_mode = mode;
    return MDG_OK;
}

MDG_API int mdg_launch_stage(mdg_system *s, int stage, unsigned mask) {
    int rc = check_sys(s);
    if (rc) return rc;
    if (!s->evaluated_once)
        return fail(MDG_ERR_STATE, "evaluate the system once before launching single stages");
    mask &= MDG_MASK_ALL;
    switch (stage) {
        case MDG_STAGE_PACK: CK(launch_pack(s), "pack"); break;
        case MDG_STAGE_NONBONDED: CK(launch_nonbonded(s, mask, 0, 0), "nonbonded"); break;
        case MDG_STAGE_NONBONDED_ENERGY:
            CK(launch_nonbonded(s, mask, 1, 0), "nonbonded with energies");
            break;
        case MDG_STAGE_SPECIAL: CK(launch_special(s, mask, 0, 0), "special"); break;
        case MDG_STAGE_PME: {
            if (!s->pme.on) return fail(MDG_ERR_STATE, "PME is not configured");
            int cr = 0;
            cudaError_t e = launch_pme(s, 0, &cr);
            if (cr != CUFFT_SUCCESS) return fail(MDG_ERR_CUFFT, "cuFFT execution failed (%d)", cr);
            CK(e, "pme");
            break;
        }
        case MDG_STAGE_BONDED: CK(launch_bonded(s, mask, 0), "bonded"); break;
        case MDG_STAGE_REORDER: CK(launch_reorder(s), "reorder"); break;
        case MDG_STAGE_INTEGRATE:
            if (s->integ_kind < 0) return fail(MDG_ERR_STATE, "integrator not configured");
            CK(launch_integrate_pre(s), "pre");
            CK(launch_integrate_post(s, 0), "post");
            break;
        default: return fail(MDG_ERR_INVALID, "unknown stage %d", stage);
    }
    if (stage != MDG_STAGE_REORDER && stage != MDG_STAGE_INTEGRATE) s->forces_valid = 0;
    return MDG_OK;
}

MDG_API int mdg_launch_count(mdg_system *s, int64_t *count) {
    if (!s) return fail(MDG_ERR_INVALID, "null system");
    if (count) *count = s->launches;
    return MDG_OK;
}

}  // extern "C"
