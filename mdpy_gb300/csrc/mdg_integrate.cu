// mdg_integrate.cu -- FP64 position/velocity update, kinetic energy, and the
// thermostat's counter-based random numbers.
//
// Replaces VerletIntegrator.integrate (mdpy/integrator/verlet_integrator.py:20-48)
// and LangevinIntegrator.integrate (mdpy/integrator/langevin_integrator.py:37-71)
// plus Ensemble._update_kinetic_energy (mdpy/ensemble.py:63-71).
//
// Both integrators are written as one "pre-force" and one "post-force" kernel
// around a single force evaluation per step:
//   pre :  x += b dt v + b dt^2/(2m) F_n + b dt/(2m) beta
//          v  = a v + a dt/(2m) F_n + b/m beta
//   post:  v += dt/(2m) F_{n+1}
// with beta = sqrt(2 m gamma kT dt) xi, a = (1-gamma dt/2)/(1+gamma dt/2),
// b = 1/(1+gamma dt/2) -- the Groenbech-Jensen--Farago scheme that mdpy's
// LangevinIntegrator writes out (with its force sign flipped and three force
// evaluations per step); gamma = 0 gives velocity Verlet.  x and v are FP64.
//
// Noise: Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11), counter =
// (atom, step_lo, step_hi, 'LANG'), key = seed; Box-Muller in float32.  The
// stream depends only on (seed, atom, step): bit-reproducible, independent
// of launch shape and of the atom sort order.
#include "mdg_internal.cuh"

namespace mdg {
namespace {

__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

__device__ __forceinline__ float3 gauss3(unsigned atom, unsigned long long step,
                                         unsigned long long seed) {
    const uint4 r = philox4x32(make_uint4(atom, (unsigned)step, (unsigned)(step >> 32), 0x4C414E47u),
                               make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const float s = 5.9604644775390625e-8f;  // 2^-24
    const float u0 = ((float)(r.x >> 8) + 0.5f) * s, u1 = ((float)(r.y >> 8) + 0.5f) * s;
    const float u2 = ((float)(r.z >> 8) + 0.5f) * s, u3 = ((float)(r.w >> 8) + 0.5f) * s;
    const float twopi = 6.28318530717958647692f;
    const float r0 = sqrtf(-2.0f * logf(u0)), r1 = sqrtf(-2.0f * logf(u2));
    return make_float3(r0 * cosf(twopi * u1), r0 * sinf(twopi * u1), r1 * cosf(twopi * u3));
}

struct InArgs {
    double *__restrict__ x;
    double *__restrict__ v;
    const double *__restrict__ mass;
    const double *__restrict__ inv_mass;
    const int *__restrict__ inv_perm;
    const unsigned long long *__restrict__ f;
    int n, n_pad;
    double dt, ca, cb, noise;  // noise = sqrt(2 gamma kT dt)
    int langevin;
    unsigned long long seed;
    unsigned long long *step;
    long long *energy;
    int *status;
    const int *__restrict__ atom_sys;
};

__device__ __forceinline__ double fget(const unsigned long long *f, int k) {
    return (double)(long long)f[k] * kFixInv;
}

// the pre-force update of atom i (cluster slot k) from the forces in slot k
__device__ __forceinline__ void pre_kick(const InArgs &a, int i, int k) {
    const double im = a.inv_mass[i];
    const double F[3] = {fget(a.f, k), fget(a.f, a.n_pad + k), fget(a.f, 2 * a.n_pad + k)};
    double bt[3] = {0.0, 0.0, 0.0};
    if (a.langevin) {
        const float3 g = gauss3((unsigned)i, *a.step, a.seed);
        const double sm = sqrt(a.mass[i]) * a.noise;
        bt[0] = sm * g.x;
        bt[1] = sm * g.y;
        bt[2] = sm * g.z;
    }
    const double h = 0.5 * a.dt * im;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double v0 = a.v[3 * i + d];
        // b dt v + b dt^2/(2m) F + b dt/(2m) beta   (h = dt/(2m))
        const double xn = a.x[3 * i + d] + a.cb * (a.dt * (v0 + h * F[d]) + h * bt[d]);
        const double vn = a.ca * v0 + a.ca * h * F[d] + a.cb * im * bt[d];
        ok = ok && isfinite(xn) && isfinite(vn);
        a.x[3 * i + d] = xn;
        a.v[3 * i + d] = vn;
    }
    if (!ok) raise_status(a.status, MDG_ERR_PARTICLE_LOSS);
}

__global__ void __launch_bounds__(256) k_pre(InArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    pre_kick(a, i, a.inv_perm[i]);
}


template <bool ENERGY>
__global__ void __launch_bounds__(256) k_post(InArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0;
    if (i < a.n) {
        const int k = a.inv_perm[i];
        const double h = 0.5 * a.dt * a.inv_mass[i];
        double vv = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double vn = a.v[3 * i + d] + h * fget(a.f, d * a.n_pad + k);
            a.v[3 * i + d] = vn;
            vv += vn * vn;
        }
        ke = 0.5 * a.mass[i] * vv;
    }
    if (i == 0) *a.step += 1ull;
    if (ENERGY) {
        const double v[1] = {ke};
        const int slot[1] = {kSlotKinetic};
        block_energy_add<1>(a.energy, i < a.n ? a.atom_sys[i] : -1, v, slot);
    }
}

__global__ void __launch_bounds__(256) k_kinetic(const double *__restrict__ v,
                                                 const double *__restrict__ mass, int n,
                                                 const int *__restrict__ atom_sys,
                                                 long long *__restrict__ energy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0;
    if (i < n) ke = 0.5 * mass[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                                     v[3 * i + 2] * v[3 * i + 2]);
    const double e[1] = {ke};
    const int slot[1] = {kSlotKinetic};
    block_energy_add<1>(energy, i < n ? atom_sys[i] : -1, e, slot);
}

__global__ void k_forces_out(const unsigned long long *__restrict__ f,
                             const int *__restrict__ inv_perm, int n, int n_pad,
                             double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = inv_perm[i];
    out[3 * i] = fget(f, k);
    out[3 * i + 1] = fget(f, n_pad + k);
    out[3 * i + 2] = fget(f, 2 * n_pad + k);
}

// mdpy's wrap_positions (mdpy/utils/pbc.py:28-36): x - L round(x * inv) with
// inv = float32(1/L) as mdpy stores pbc_inv (mdpy/core/state.py:53-54), so an
// exact half-box coordinate lands on the side mdpy puts it
__global__ void k_positions_out(const double *__restrict__ x, int n,
                                const SysDev *__restrict__ sys, const int *__restrict__ atom_sys,
                                double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *L = sys[atom_sys[i]].Ld;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double p = x[3 * i + d];
        const double inv32 = (double)(float)(1.0 / L[d]);
        out[3 * i + d] = p - L[d] * rint(p * inv32);
    }
}

__global__ void k_noise(int n, unsigned long long step, unsigned long long seed, float *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 g = gauss3((unsigned)i, step, seed);
    out[3 * i] = g.x;
    out[3 * i + 1] = g.y;
    out[3 * i + 2] = g.z;
}

// one steepest-descent move (SteepestDescentMinimizer.minimize,
// mdpy/minimizer/steepest_descent_minimizer.py:39-42): every atom moves
// alpha A along its own force direction.  An atom with zero force stays put
// (the reference divides by the zero norm).
__global__ void __launch_bounds__(256) k_sd_step(double *__restrict__ x,
                                                 const unsigned long long *__restrict__ f,
                                                 const int *__restrict__ inv_perm, int n,
                                                 int n_pad, double alpha,
                                                 int *__restrict__ status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = inv_perm[i];
    const double F[3] = {fget(f, k), fget(f, n_pad + k), fget(f, 2 * n_pad + k)};
    const double norm = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
    if (!(norm > 0.0)) return;
    const double c = alpha / norm;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double xn = x[3 * i + d] + c * F[d];
        ok = ok && isfinite(xn);
        x[3 * i + d] = xn;
    }
    if (!ok) raise_status(status, MDG_ERR_PARTICLE_LOSS);
}

InArgs make_args(mdg_system *s) {
    InArgs a;
    a.x = s->x;
    a.v = s->v;
    a.mass = s->mass;
    a.inv_mass = s->inv_mass;
    a.inv_perm = s->inv_perm;
    a.f = s->f;
    a.n = s->n;
    a.n_pad = s->n_pad;
    a.dt = s->dt;
    const bool lg = s->integ_kind == MDG_INTEGRATOR_LANGEVIN && s->friction > 0;
    const double g = lg ? s->friction : 0.0;
    a.ca = (1.0 - 0.5 * g * s->dt) / (1.0 + 0.5 * g * s->dt);
    a.cb = 1.0 / (1.0 + 0.5 * g * s->dt);
    // kB in mdpy's internal units (J/K / (Da A^2 fs^-2)), same inputs as mdpy/unit/__init__.py:54
    const double kB = 1.38064852e-23 / (1.66053904e-27 * 1e-20 / 1e-30);
    a.noise = lg ? sqrt(2.0 * g * kB * s->temperature * s->dt) : 0.0;
    a.langevin = lg ? 1 : 0;
    a.seed = s->seed;
    a.step = s->step_dev;
    a.energy = s->energy;
    a.status = s->status;
    a.atom_sys = s->atom_sys;
    return a;
}

}  // namespace

cudaError_t launch_integrate_pre(mdg_system *s) {
    InArgs a = make_args(s);
    k_pre<<<(s->n + 255) / 256, 256, 0, s->stream>>>(a);
    s->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_integrate_post(mdg_system *s, int energy) {
    InArgs a = make_args(s);
    if (energy)
        k_post<true><<<(s->n + 255) / 256, 256, 0, s->stream>>>(a);
    else
        k_post<false><<<(s->n + 255) / 256, 256, 0, s->stream>>>(a);
    s->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_kinetic(mdg_system *s) {
    k_kinetic<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->v, s->mass, s->n, s->atom_sys,
                                                         s->energy);
    s->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_forces_out(mdg_system *s) {
    k_forces_out<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->f, s->inv_perm, s->n, s->n_pad,
                                                            s->fout);
    s->launches += 1;
    return cudaGetLastError();
}

// flag |= 1 unless xin equals, bit for bit, what k_positions_out reports for x
__global__ void k_same_positions(const double *__restrict__ x, int n,
                                 const SysDev *__restrict__ sys, const int *__restrict__ atom_sys,
                                 const double *__restrict__ xin, int *flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool differ = false;
    if (i < n) {
        const double *L = sys[atom_sys[i]].Ld;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double p = x[3 * i + d];
            const double inv32 = (double)(float)(1.0 / L[d]);
            differ |= xin[3 * i + d] != p - L[d] * rint(p * inv32);
        }
    }
    if (__any_sync(0xffffffffu, differ) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

cudaError_t launch_same_positions(mdg_system *s, const double *xin, int *flag) {
    k_same_positions<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->x, s->n, s->sys_dev,
                                                                 s->atom_sys, xin, flag);
    s->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_positions_out(mdg_system *s, double *out) {
    k_positions_out<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->x, s->n, s->sys_dev,
                                                                s->atom_sys, out);
    s->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_sd_step(mdg_system *s, double alpha) {
    k_sd_step<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->x, s->f, s->inv_perm, s->n, s->n_pad,
                                                         alpha, s->status);
    s->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_noise(mdg_system *s, uint64_t step, float *out) {
    k_noise<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->n, step, s->seed, out);
    s->launches += 1;
    return cudaGetLastError();
}

}  // namespace mdg
