// mdg_nonbonded.cu -- short-range nonbonded forces.
//
// Replaces, for the pair work:
//   CharmmNonbondedConstraint.cpu_kernel / cuda_kernel
//     (mdpy/constraint/charmm_nonbonded_constraint.py:64-181): LJ 12-6 with
//     Lorentz-Berthelot combination, 1-4 parameters for scaling_particles,
//     bonded_particles excluded, hard cutoff r <= rc;
//   ElectrostaticConstraint (mdpy/constraint/electrostatic_constraint.py:52-135):
//     bare Coulomb, all pairs, minimum image (kept as MDG_COUL_BARE for parity);
// and adds the Ewald real-space term k q_i q_j erfc(beta r)/r (MDG_COUL_EWALD),
// which mdpy v0.2.1 does not have, plus an optional CHARMM switch for LJ.
//
// Design (GB300): `split` (default 4) independent single-warp work items per 32-atom
// i-cluster I (no block barrier: a warp that finishes early frees its slot).
//   1. each warp walks its own interleaved batches of cluster bounding boxes
//      (a balanced half shell: the cluster pair {I, J} belongs to one of the
//      two by the parity of I + J) and takes every (J, periodic image) whose
//      box lies within rc of I's box -- __ballot_sync over 32 clusters at a
//      time, no candidate list and no block barrier;
//   2. for each candidate every lane tests one j atom against I's bounding
//      box, and the survivors are appended (warp ballot + popc, no atomics)
//      to a 64-entry per-warp ring buffer in shared memory, already shifted
//      to the right periodic image and with a 32-bit exclusion mask (which i
//      lanes must skip this j);
//   3. each full chunk of 32 j entries is swept against the warp's 32 i atoms
//      in 32 rotation steps: at step t lane l pairs its i atom with entry
//      (l+t) mod 32, keeps the i force in registers and passes the j force
//      accumulator to lane l-1 with one shuffle per component, so after the
//      sweep every lane owns one entry's complete j force.  No shared-memory
//      atomics, no per-pair reduction trees.
// Forces leave as int64 fixed point (scale 2^32) through 64-bit global
// atomics: the sum is independent of the order of arrival, so results are
// bit-reproducible run to run.  Pairs are never stored: the pair set is
// found afresh from the current coordinates on every evaluation, so no
// Verlet skin or rebuild criterion exists that could miss a pair.
#include <algorithm>

#include "mdg_nonbonded_kernel.cuh"

namespace mdg {

cudaError_t launch_nb_half(mdg_system *s, const NbArgs &a, int coul_tile, bool want_lj, bool sw,
                           int energy, int dump);  // mdg_nonbonded_half.cu
cudaError_t launch_nb_quarter(mdg_system *s, const NbArgs &a, int coul_tile, bool want_lj,
                              bool sw, int energy, int dump);  // mdg_nonbonded_quarter.cu

namespace {

// Bare Coulomb over all pairs with the minimum image (parity path for
// ElectrostaticConstraint, electrostatic_constraint.py:52-79): one thread per
// i atom, j atoms staged through shared memory in tiles, forces on i only.
__global__ void __launch_bounds__(256) k_coulomb_bare(NbArgs a) {
    __shared__ float4 s_x[256];
    // sorted slots, padding included; uncharged slots (padding has q = 0)
    // contribute nothing and are skipped; j runs over i's own system only
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float4 xi = i < a.n_pad ? a.xq[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool iv = i < a.n_pad && xi.w != 0.f;
    const int sid = i < a.n_pad ? a.cl_sys[i / kCluster] : -1;
    float L[3] = {1.f, 1.f, 1.f}, invL[3] = {1.f, 1.f, 1.f};
    if (sid >= 0) {
        const SysDev &sd = a.sys[sid];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            L[k] = sd.L[k];
            invL[k] = sd.invL[k];
        }
    }
    float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
    for (int base = 0; base < a.n_pad; base += 256) {
        const int jl = base + threadIdx.x;
        s_x[threadIdx.x] = jl < a.n_pad ? a.xq[jl] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        const int lim = min(256, a.n_pad - base);
        if (iv) {
            for (int t = 0; t < lim; ++t) {
                const int j = base + t;
                if (j == i || s_x[t].w == 0.f) continue;
                if (a.cl_sys[j / kCluster] != sid) continue;
                bool excl = false;
                for (int w = 0; w < a.pw; ++w) {
                    const int p = a.partners[(size_t)i * a.pw + w];
                    if (p >= 0 && !(p & 0x40000000) && p == j) excl = true;
                }
                if (excl) continue;
                const float4 xj = s_x[t];
                float d[3] = {xj.x - xi.x, xj.y - xi.y, xj.z - xi.z};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float sc = d[k] * invL[k];
                    d[k] = (sc - rintf(sc)) * L[k];
                }
                const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                const float rinv = rsqrtf(r2);
                const float qq = xi.w * xj.w;
                const float ev = qq * rinv;
                const float fr = ev * rinv * rinv;
                e += 0.5f * ev;
                fx -= fr * d[0];
                fy -= fr * d[1];
                fz -= fr * d[2];
            }
        }
        __syncthreads();
    }
    if (iv) {
        fix_red(&a.f[i], to_fix(fx));
        fix_red(&a.f[a.n_pad + i], to_fix(fy));
        fix_red(&a.f[2 * a.n_pad + i], to_fix(fz));
    }
    const double v[1] = {(double)e};
    const int slot[1] = {MDG_TERM_COUL_REAL};
    block_energy_add<1>(a.energy, iv ? sid : -1, v, slot);
}

// ---- special pairs ---------------------------------------------------------
struct SpArgs {
    const double *__restrict__ x;
    const int *__restrict__ inv_perm;
    const float *__restrict__ charge;  // q * sqrt(k_e), atom order
    const float4 *__restrict__ lj;     // atom order
    const int2 *__restrict__ excl;
    const int2 *__restrict__ p14;
    const SysDev *__restrict__ sys;
    const int *__restrict__ atom_sys;
    int n_excl, n_14, n_pad;
    float rc, rc2, rs2, sw_inv_den, beta, ewald_fc;
    int do_excl, do_lj14, do_coul14;
    float excl_weight;  // weight of the excluded-pair reciprocal correction's force
    unsigned long long *f;
    unsigned long long *fx;  // where the excluded-pair correction's force goes
    long long *energy;
    int *dump;
    long long dump_cap;
    unsigned long long *dump_count;
};

// Excluded 1-2/1-3 pairs: -k q q erf(beta r)/r removes their share of the
// reciprocal sum (term COUL_RECIP).  1-4 pairs: LJ with the 1-4 parameters
// (charmm_nonbonded_constraint.py:92-97) and the real-space Coulomb term.
template <bool SWITCH, bool DUMP>
__global__ void k_special(SpArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    float e_lj = 0.f, e_cr = 0.f, e_rec = 0.f;
    int sid = -1;
    if (t < a.n_excl + a.n_14) {
        const bool is14 = t >= a.n_excl;
        const int2 pr = is14 ? a.p14[t - a.n_excl] : a.excl[t];
        const int i = pr.x, j = pr.y;
        sid = a.atom_sys[i];
        const SysDev &sd = a.sys[sid];
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double dd = a.x[3 * j + k] - a.x[3 * i + k];
            dd -= sd.Ld[k] * rint(dd * sd.invLd[k]);
            d[k] = (float)dd;
        }
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const float r = sqrtf(r2);
        const float qq = a.charge[i] * a.charge[j];
        float fr = 0.f;
        if (!is14) {
            if (a.do_excl) {
                const float br = a.beta * r;
                const float ef = erff(br);
                e_rec = -qq * ef / r;
                fr = a.excl_weight * qq * (a.ewald_fc * expf(-br * br) * r - ef) / (r2 * r);
            }
        } else if (DUMP) {
            // pair dump: the reference's own float32 pair test decides
            if (ref_within32(a.x, i, j, sd, a.rc)) {
                unsigned long long slot = atomicAdd(a.dump_count, 1ull);
                if ((long long)slot < a.dump_cap) {
                    a.dump[2 * slot] = min(i, j);
                    a.dump[2 * slot + 1] = max(i, j);
                }
            }
        } else if (r2 <= a.rc2) {
            if (a.do_lj14) {
                const float4 pi = a.lj[i], pj = a.lj[j];
                const float sig = pi.z + pj.z;
                const float s2 = sig * sig / r2;
                const float s6 = s2 * s2 * s2;
                const float c6 = pi.w * pj.w * s6;
                float elj = c6 * (s6 - 1.0f);
                float flj = c6 * (12.0f * s6 - 6.0f) / r2;
                if (SWITCH && r2 > a.rs2) {
                    const float u = a.rc2 - r2;
                    const float sw = u * u * (a.rc2 + 2.0f * r2 - 3.0f * a.rs2) * a.sw_inv_den;
                    const float dsw = 12.0f * u * (a.rs2 - r2) * a.sw_inv_den;
                    flj = flj * sw - elj * dsw;
                    elj *= sw;
                }
                e_lj = elj;
                fr += flj;
            }
            if (a.do_coul14) {
                const float br = a.beta * r;
                const float ec = erfcf(br);
                e_cr = qq * ec / r;
                fr += qq * (ec / r + a.ewald_fc * expf(-br * br)) / r2;
            }
        }
        if (!DUMP && fr != 0.f) {
            const int ki = a.inv_perm[i], kj = a.inv_perm[j];
            unsigned long long *ff = is14 ? a.f : a.fx;
            fix_red(&ff[kj], to_fix(fr * d[0]));
            fix_red(&ff[a.n_pad + kj], to_fix(fr * d[1]));
            fix_red(&ff[2 * a.n_pad + kj], to_fix(fr * d[2]));
            fix_red(&ff[ki], to_fix(-fr * d[0]));
            fix_red(&ff[a.n_pad + ki], to_fix(-fr * d[1]));
            fix_red(&ff[2 * a.n_pad + ki], to_fix(-fr * d[2]));
        }
    }
    if (DUMP) return;
    // FP64 block sums: the exclusion term is a sum of O(10^5) terms of either
    // sign whose total largely cancels the self energy
    const double v[3] = {(double)e_lj, (double)e_cr, (double)e_rec};
    const int slot[3] = {MDG_TERM_LJ, MDG_TERM_COUL_REAL, MDG_TERM_COUL_RECIP};
    block_energy_add<3>(a.energy, sid, v, slot);
}

NbArgs make_args(mdg_system *s) {
    NbArgs a;
    a.xq = s->xq;
    a.prm = s->prm_sorted;
    a.partners = s->partners_sorted;
    a.pw = s->pw;
    a.prange = s->cluster_partner_range;
    a.bbox = s->bbox;
    a.n = s->n;
    a.n_pad = s->n_pad;
    a.n_clusters = s->n_clusters;
    a.sys = s->sys_dev;
    a.cl_sys = s->cl_sys;
    a.cl_col = s->cl_col;
    a.hbox = s->hbox;
    a.qbox = s->qbox;
    a.col_xy = s->col_xy;
    a.col_rank = s->cell_rank;
    a.col_cl_start = s->col_cl_start;
    a.col_ncl = s->col_ncl;
    a.overhang = s->overhang;
    a.rc = s->cutoff;
    a.rc2 = s->cutoff * s->cutoff;
    const double rs = s->rswitch > 0 ? s->rswitch : s->cutoff;
    a.rs2 = (float)(rs * rs);
    const double den = (double)a.rc2 - rs * rs;
    a.sw_inv_den = den > 0 ? (float)(1.0 / (den * den * den)) : 0.f;
    a.sw_um = den > 0 ? (float)(-1.0 / den) : 0.f;
    a.sw_uc = den > 0 ? (float)((double)a.rc2 / den) : 1.f;
    a.sw_g = den > 0 ? (float)(12.0 / den) : 0.f;
    a.beta = (float)s->beta;
    a.beta_p = kAsP * (float)s->beta;
    a.ewald_exp_c = (float)(s->beta * s->beta * 1.4426950408889634);
    a.ewald_fc = (float)(2.0 * s->beta / 1.7724538509055159);
    a.lj_on = s->lj_on;
    a.f = s->f;
    a.energy = s->energy;
    a.status = s->status;
    a.stats = s->stats;
    a.dump = s->dump_buf;
    a.dump_cap = s->dump_cap;
    a.dump_count = s->dump_count;
    a.perm = s->perm;
    a.x = s->x;
    a.rc_ref = s->cutoff;
    a.split = s->nb_split;
    a.persistent = s->nb_persistent > 0;
    a.n_items = s->n_clusters * s->nb_split;
    a.queue = s->nb_queue;
    // persistent form: one queue atomic per `grab` consecutive items, so
    // that a batch of ~10^5 items does not serialise on the counter; each
    // resident warp still sees about 16 grabs, which keeps the tail short
    a.grab = 1;
    if (s->nb_persistent_ctas > 0)
        a.grab = std::max(1, std::min(8, a.n_items / (16 * s->nb_persistent_ctas)));
    a.split_rings = s->nb_split_rings;
    return a;
}


}  // namespace

cudaError_t launch_nonbonded(mdg_system *s, unsigned mask, int energy, int dump) {
    const bool want_lj = (mask & MDG_MASK(MDG_TERM_LJ)) && s->lj_on;
    const bool want_c = (mask & MDG_MASK(MDG_TERM_COUL_REAL)) && s->coul_mode != MDG_COUL_NONE;
    if (!want_lj && !want_c) return cudaSuccess;
    NbArgs a = make_args(s);
    a.lj_on = want_lj ? 1 : 0;
    if (dump) {
        // the pair dump searches a little beyond the cutoff and lets the
        // reference's float32 test (ref_within32) decide each candidate:
        // the packed float32 coordinates differ from the reference's by
        // rounding (~1e-5 A), far below this margin
        a.rc = s->cutoff + kDumpMargin;
        a.rc2 = a.rc * a.rc;
    }
    const bool sw = s->rswitch > 0 && s->rswitch < s->cutoff;
    cudaError_t err = cudaSuccess;
    const int coul_tile = (want_c && s->coul_mode == MDG_COUL_EWALD) ? MDG_COUL_EWALD : MDG_COUL_NONE;
    if (want_lj || coul_tile == MDG_COUL_EWALD) {
        err = s->nb_half == 2   ? launch_nb_quarter(s, a, coul_tile, want_lj, sw, energy, dump)
              : s->nb_half == 1 ? launch_nb_half(s, a, coul_tile, want_lj, sw, energy, dump)
                                : dispatch_shape<false>(s, a, coul_tile, want_lj, sw, energy, dump);
        s->launches += 1;
        if (err != cudaSuccess) return err;
    }
    if (want_c && s->coul_mode == MDG_COUL_BARE && !dump) {
        k_coulomb_bare<<<(s->n_pad + 255) / 256, 256, 0, s->stream>>>(a);
        s->launches += 1;
        err = cudaGetLastError();
    }
    return err;
}

cudaError_t launch_special(mdg_system *s, unsigned mask, int energy, int dump) {
    (void)energy;
    SpArgs a;
    a.x = s->x;
    a.inv_perm = s->inv_perm;
    a.charge = s->charge;
    a.lj = s->lj;
    a.excl = s->excl_pairs;
    a.p14 = s->pairs14;
    a.n_excl = s->n_excl;
    a.n_14 = s->n_14;
    a.n_pad = s->n_pad;
    a.sys = s->sys_dev;
    a.atom_sys = s->atom_sys;
    a.rc = s->cutoff;
    a.rc2 = s->cutoff * s->cutoff;
    const double rs = s->rswitch > 0 ? s->rswitch : s->cutoff;
    a.rs2 = (float)(rs * rs);
    const double den = (double)a.rc2 - rs * rs;
    a.sw_inv_den = den > 0 ? (float)(1.0 / (den * den * den)) : 0.f;
    a.beta = (float)s->beta;
    a.ewald_fc = (float)(2.0 * s->beta / 1.7724538509055159);
    a.do_excl = (mask & MDG_MASK(MDG_TERM_COUL_RECIP)) && s->pme.on && !dump;
    a.excl_weight = s->recip_weight;
    a.do_lj14 = (mask & MDG_MASK(MDG_TERM_LJ)) && s->lj_on;
    a.do_coul14 = (mask & MDG_MASK(MDG_TERM_COUL_REAL)) && s->coul_mode == MDG_COUL_EWALD;
    a.f = s->f;
    a.fx = s->slow_target ? s->slow_target : s->f;
    a.energy = s->energy;
    a.dump = s->dump_buf;
    a.dump_cap = s->dump_cap;
    a.dump_count = s->dump_count;
    if (!dump && !a.do_lj14 && !a.do_coul14) a.n_14 = 0;
    if (!a.do_excl) a.n_excl = 0;
    if (dump && !(a.do_lj14 || a.do_coul14)) a.n_14 = 0;
    const int total = a.n_excl + a.n_14;
    if (total == 0) return cudaSuccess;
    const bool sw = s->rswitch > 0 && s->rswitch < s->cutoff;
    const int tb = 256, nb = (total + tb - 1) / tb;
    if (dump)
        sw ? k_special<true, true><<<nb, tb, 0, s->stream>>>(a)
           : k_special<false, true><<<nb, tb, 0, s->stream>>>(a);
    else
        sw ? k_special<true, false><<<nb, tb, 0, s->stream>>>(a)
           : k_special<false, false><<<nb, tb, 0, s->stream>>>(a);
    s->launches += 1;
    return cudaGetLastError();
}

}  // namespace mdg
