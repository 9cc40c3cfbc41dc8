// mdg_bonded.cu -- CHARMM bonded terms, one thread per term.
//
// Replaces the numba loops of
//   CharmmBondConstraint.kernel     V = k (r - r0)^2
//                                   (mdpy/constraint/charmm_bond_constraint.py:52-73)
//   CharmmAngleConstraint.kernel    V = k (theta - theta0)^2 + ku (r13 - u0)^2
//                                   (mdpy/constraint/charmm_angle_constraint.py:138-179)
//   CharmmDihedralConstraint.kernel V = k (1 + cos(n phi - delta))
//                                   (mdpy/constraint/charmm_dihedral_constraint.py:58-95)
//   CharmmImproperConstraint.kernel V = k (psi - psi0)^2
//                                   (mdpy/constraint/charmm_improper_constraint.py:56-93)
// with the same energy conventions (no factor 1/2) and dihedral angle
// definition (get_pbc_dihedral, mdpy/utils/geometry.py:73-86).  The forces are
// the exact negative gradients (torsion derivative of Blondel & Karplus 1996);
// the reference's dihedral force at charmm_dihedral_constraint.py:81 is not
// -dV/dphi and is deliberately not reproduced.
//
// Differences are taken in FP64 from the FP64 state (minimum image), the term
// arithmetic is FP32, and forces go to the int64 fixed-point accumulators.
// One launch covers all four term types: the grid is split into segments of
// whole blocks per type, so each block reduces a single energy term.
#include "mdg_internal.cuh"

namespace mdg {
namespace {

struct BdArgs {
    const double *__restrict__ x;
    const int *__restrict__ inv_perm;
    const SysDev *__restrict__ sys;
    const int *__restrict__ atom_sys;
    const int2 *__restrict__ bidx;
    const float2 *__restrict__ bprm;
    const int4 *__restrict__ aidx;
    const float4 *__restrict__ aprm;
    const int4 *__restrict__ didx;
    const float4 *__restrict__ dprm;
    const int4 *__restrict__ iidx;
    const float2 *__restrict__ iprm;
    int nb, na, nd, ni;
    int blk[4];  // first block of each segment (bond, angle, dihedral, improper) + end
    int blk_end;
    unsigned long long *f;
    int n_pad;
    long long *energy;
};

__device__ __forceinline__ float3 mind(const BdArgs &a, int i, int j) {
    const SysDev &sd = a.sys[a.atom_sys[i]];  // a term never spans two systems
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        d[k] = a.x[3 * j + k] - a.x[3 * i + k];
        d[k] -= sd.Ld[k] * rint(d[k] * sd.invLd[k]);
    }
    return make_float3((float)d[0], (float)d[1], (float)d[2]);
}

__device__ __forceinline__ void addf(const BdArgs &a, int atom, float fx, float fy, float fz) {
    const int k = a.inv_perm[atom];
    fix_red(&a.f[k], to_fix(fx));
    fix_red(&a.f[a.n_pad + k], to_fix(fy));
    fix_red(&a.f[2 * a.n_pad + k], to_fix(fz));
}

__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// dihedral angle (get_pbc_dihedral) and its gradient g[4] w.r.t. the 4 atoms
__device__ float torsion(const BdArgs &a, int4 id, float3 g[4], bool &ok) {
    const float3 b1 = mind(a, id.x, id.y), b2 = mind(a, id.y, id.z), b3 = mind(a, id.z, id.w);
    const float3 m = cross(b1, b2), n = cross(b2, b3);
    const float lb2 = sqrtf(dot(b2, b2));
    const float phi = atan2f(lb2 * dot(b1, n), dot(m, n));
    const float m2 = dot(m, m), n2 = dot(n, n);
    ok = m2 > 1e-20f && n2 > 1e-20f && lb2 > 1e-10f;
    if (!ok) return phi;
    const float cm = -lb2 / m2, cn = lb2 / n2;
    g[0] = make_float3(cm * m.x, cm * m.y, cm * m.z);
    g[3] = make_float3(cn * n.x, cn * n.y, cn * n.z);
    const float p = dot(b1, b2) / (lb2 * lb2), r = dot(b3, b2) / (lb2 * lb2);
    g[1] = make_float3(-(1 + p) * g[0].x + r * g[3].x, -(1 + p) * g[0].y + r * g[3].y,
                       -(1 + p) * g[0].z + r * g[3].z);
    g[2] = make_float3(p * g[0].x - (1 + r) * g[3].x, p * g[0].y - (1 + r) * g[3].y,
                       p * g[0].z - (1 + r) * g[3].z);
    return phi;
}

__global__ void __launch_bounds__(256) k_bonded(BdArgs a) {
    const int b = blockIdx.x;
    int seg = 0;
    while (seg < 3 && b >= a.blk[seg + 1]) ++seg;
    const int t = (b - a.blk[seg]) * blockDim.x + threadIdx.x;
    float e = 0.f;
    int first = -1;  // first atom of this thread's term
    if (seg == 0 && t < a.nb) {
        const int2 id = a.bidx[t];
        first = id.x;
        const float2 p = a.bprm[t];
        const float3 d = mind(a, id.x, id.y);
        const float r = sqrtf(dot(d, d));
        const float dr = r - p.y;
        e = p.x * dr * dr;
        const float fr = 2.f * p.x * dr / r;  // force on i along +d
        addf(a, id.x, fr * d.x, fr * d.y, fr * d.z);
        addf(a, id.y, -fr * d.x, -fr * d.y, -fr * d.z);
    } else if (seg == 1 && t < a.na) {
        const int4 id = a.aidx[t];
        first = id.x;
        const float4 p = a.aprm[t];
        const float3 u = mind(a, id.y, id.x), w = mind(a, id.y, id.z);  // r21, r23
        const float lu = sqrtf(dot(u, u)), lw = sqrtf(dot(w, w));
        float c = dot(u, w) / (lu * lw);
        c = fminf(fmaxf(c, -1.f), 1.f);
        const float th = acosf(c);
        const float s = fmaxf(sqrtf(fmaxf(1.f - c * c, 0.f)), 1e-6f);
        const float dth = th - p.y;
        e = p.x * dth * dth;
        const float dv = 2.f * p.x * dth;
        const float iul = 1.f / (lu * lw), iu2 = 1.f / (lu * lu), iw2 = 1.f / (lw * lw);
        // dtheta/dx_i = -(w/(lu lw) - c u/lu^2)/s ; dtheta/dx_l = -(u/(lu lw) - c w/lw^2)/s
        const float3 gi = make_float3(-(w.x * iul - c * u.x * iu2) / s, -(w.y * iul - c * u.y * iu2) / s,
                                      -(w.z * iul - c * u.z * iu2) / s);
        const float3 gl = make_float3(-(u.x * iul - c * w.x * iw2) / s, -(u.y * iul - c * w.y * iw2) / s,
                                      -(u.z * iul - c * w.z * iw2) / s);
        float3 fi = make_float3(-dv * gi.x, -dv * gi.y, -dv * gi.z);
        float3 fl = make_float3(-dv * gl.x, -dv * gl.y, -dv * gl.z);
        float3 fj = make_float3(-(fi.x + fl.x), -(fi.y + fl.y), -(fi.z + fl.z));
        if (p.z != 0.f) {  // Urey-Bradley 1-3 term
            const float3 d = mind(a, id.x, id.z);
            const float r = sqrtf(dot(d, d));
            const float dr = r - p.w;
            e += p.z * dr * dr;
            const float fr = 2.f * p.z * dr / r;
            fi.x += fr * d.x;
            fi.y += fr * d.y;
            fi.z += fr * d.z;
            fl.x -= fr * d.x;
            fl.y -= fr * d.y;
            fl.z -= fr * d.z;
        }
        addf(a, id.x, fi.x, fi.y, fi.z);
        addf(a, id.y, fj.x, fj.y, fj.z);
        addf(a, id.z, fl.x, fl.y, fl.z);
    } else if ((seg == 2 && t < a.nd) || (seg == 3 && t < a.ni)) {
        const int4 id = seg == 2 ? a.didx[t] : a.iidx[t];
        first = id.x;
        float3 g[4];
        bool ok;
        const float phi = torsion(a, id, g, ok);
        float dv;
        if (seg == 2) {
            const float4 p = a.dprm[t];  // k, n, delta
            const float arg = p.y * phi - p.z;
            e = p.x * (1.f + cosf(arg));
            dv = -p.x * p.y * sinf(arg);
        } else {
            const float2 p = a.iprm[t];  // k, psi0
            float dp = phi - p.y;
            const float pi = 3.14159265358979f;
            if (dp > pi) dp -= 2.f * pi;
            if (dp < -pi) dp += 2.f * pi;
            e = p.x * dp * dp;
            dv = 2.f * p.x * dp;
        }
        if (ok) {
            addf(a, id.x, -dv * g[0].x, -dv * g[0].y, -dv * g[0].z);
            addf(a, id.y, -dv * g[1].x, -dv * g[1].y, -dv * g[1].z);
            addf(a, id.z, -dv * g[2].x, -dv * g[2].y, -dv * g[2].z);
            addf(a, id.w, -dv * g[3].x, -dv * g[3].y, -dv * g[3].z);
        }
    }
    const double v[1] = {(double)e};
    const int slot[1] = {MDG_TERM_BOND + seg};
    block_energy_add<1>(a.energy, first >= 0 ? a.atom_sys[first] : -1, v, slot);
}

}  // namespace

cudaError_t launch_bonded(mdg_system *s, unsigned mask, int energy) {
    (void)energy;
    BdArgs a;
    a.x = s->x;
    a.inv_perm = s->inv_perm;
    a.sys = s->sys_dev;
    a.atom_sys = s->atom_sys;
    a.bidx = s->bond_idx;
    a.bprm = s->bond_prm;
    a.aidx = s->angle_idx;
    a.aprm = s->angle_prm;
    a.didx = s->dih_idx;
    a.dprm = s->dih_prm;
    a.iidx = s->imp_idx;
    a.iprm = s->imp_prm;
    a.nb = (mask & MDG_MASK(MDG_TERM_BOND)) ? s->nb : 0;
    a.na = (mask & MDG_MASK(MDG_TERM_ANGLE)) ? s->na : 0;
    a.nd = (mask & MDG_MASK(MDG_TERM_DIHEDRAL)) ? s->nd : 0;
    a.ni = (mask & MDG_MASK(MDG_TERM_IMPROPER)) ? s->ni : 0;
    const int tb = 256;
    const int nblk[4] = {(a.nb + tb - 1) / tb, (a.na + tb - 1) / tb, (a.nd + tb - 1) / tb,
                         (a.ni + tb - 1) / tb};
    a.blk[0] = 0;
    for (int k = 1; k < 4; ++k) a.blk[k] = a.blk[k - 1] + nblk[k - 1];
    a.blk_end = a.blk[3] + nblk[3];
    if (a.blk_end == 0) return cudaSuccess;
    a.f = s->f;
    a.n_pad = s->n_pad;
    a.energy = s->energy;
    k_bonded<<<a.blk_end, tb, 0, s->stream>>>(a);
    s->launches += 1;
    return cudaGetLastError();
}

}  // namespace mdg
