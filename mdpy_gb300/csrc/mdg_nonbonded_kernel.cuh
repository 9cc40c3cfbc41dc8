// mdg_nonbonded_kernel.cuh -- the pair kernel's templates, shared by the
// two translation units that instantiate them (whole-warp and half-warp i
// groups), so that the library builds in parallel.
#pragma once

#include <type_traits>

#include "mdg_internal.cuh"

namespace mdg {

struct NbArgs {
    const float4 *__restrict__ xq;
    const float2 *__restrict__ prm;
    const int *__restrict__ partners;
    int pw;
    const int2 *__restrict__ prange;
    const float4 *__restrict__ bbox;
    const SysDev *__restrict__ sys;
    const int *__restrict__ cl_sys;
    const float4 *__restrict__ hbox;       // boxes of each cluster's two 16-slot halves
    const float4 *__restrict__ qbox;       // boxes of each cluster's four 8-slot quarters
    const int *__restrict__ cl_col;        // cluster -> global sort column
    const int *__restrict__ col_xy;        // global column -> (cx << 16) | cy
    const int *__restrict__ col_rank;      // system column (cx * ncy + cy) -> rank
    const int *__restrict__ col_cl_start;  // global column -> first cluster (scan)
    const int *__restrict__ col_ncl;       // global column -> clusters
    const float *__restrict__ overhang;    // per system, A
    int n, n_pad, n_clusters;
    float rc, rc2, rs2, sw_inv_den;
    float sw_um, sw_uc, sw_g;  // switch: u = r^2 sw_um + sw_uc; g = 12 / (rc^2 - rs^2)
    float beta;
    float beta_p;        // A&S p * beta
    float ewald_exp_c;   // beta^2 log2(e)
    float ewald_fc;      // 2 beta / sqrt(pi)
    int lj_on;
    unsigned long long *f;
    long long *energy;
    int *status;
    unsigned long long *stats;
    int *dump;
    long long dump_cap;
    unsigned long long *dump_count;
    const int *perm;
    const double *x;  // FP64 state, atom order (pair dump: the reference's pair test)
    float rc_ref;     // pair dump: the cutoff of that test (the search uses rc + a margin)
    int split;        // work items (one warp each) per i-cluster
    int persistent;   // 1: warps pull items from `queue` until none is left
    int n_items;      // n_clusters * split
    int *queue;       // next item (zeroed before each persistent launch)
    int grab;         // persistent form: consecutive items a warp takes per queue atomic
    int split_rings;  // 1: separate rings for LJ-carrying and charge-only j atoms
};

namespace {

constexpr int kRing = 64;
constexpr unsigned kFull = 0xffffffffu;
// the pair dump's search radius beyond the cutoff (A)
constexpr float kDumpMargin = 0.01f;

// Abramowitz & Stegun 7.1.26: erfc(x) ~ t(a1 + t(a2 + t(a3 + t(a4 + t a5)))) e^{-x^2},
// t = 1/(1 + p x), |error| <= 1.5e-7
constexpr float kAsP = 0.3275911f;
constexpr float kAsA1 = 0.254829592f, kAsA2 = -0.284496736f, kAsA3 = 1.421413741f,
                kAsA4 = -1.453152027f, kAsA5 = 1.061405429f;


__device__ __forceinline__ void decode_shift(int code, const float (&L)[3], float &sx, float &sy,
                                             float &sz) {
    sx = (float)(code / 9 - 1) * L[0];
    sy = (float)((code / 3) % 3 - 1) * L[1];
    sz = (float)(code % 3 - 1) * L[2];
}

// 2^x and 1/x as single special-function instructions (PTX ex2.approx /
// rcp.approx, flush-to-zero; relative error below 2^-22): the pair kernel's
// arguments stay in normal range (2^x with x in [-16, 0], 1/x with x in
// [1, 2.1])
__device__ __forceinline__ float fast_exp2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float fast_rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// erfc(x) for the reported real-space energy, from the two factors the
// force already has: erfc(x) = e^{-x^2} t Q(t), t = 1/(1 + p x) with the
// Abramowitz & Stegun p of the force's fit.  Q(t) is a degree-7 polynomial
// in t - kEqC fitted here (weighted least squares toward a uniform relative
// error) to erfcx(x) / t = e^{x^2} erfc(x) / t over x in [0, 6]: relative
// error 5e-8 in exact arithmetic, 4e-7 at most (8e-8 on average) evaluated
// in FP32 -- a relative fit, so the error stays small where erfc is small,
// which an absolute fit such as the force's does not (its 1.5e-7 is 5 % of
// erfc(3.3)).  x = beta r <= 6 covers Ewald tolerances down to 1e-15;
// beyond it the product is below 1e-16 of q q / r.
constexpr float kEqC = 0.668603f;
__device__ __forceinline__ float erfc_q(float t) {
    const float u = t - kEqC;
    float q = fmaf(u, -0.143815756f, -0.165253997f);
    q = fmaf(u, q, 0.262164414f);
    q = fmaf(u, q, 0.950700283f);
    q = fmaf(u, q, 1.40503132f);
    q = fmaf(u, q, 1.35223436f);
    q = fmaf(u, q, 0.93637538f);
    return fmaf(u, q, 0.477811038f);
}

// One j entry staged in shared memory, two float4: the shifted coordinates
// + charge, and (sigma/2, sqrt(4 eps), exclusion mask of the 32 i lanes,
// cluster-order index) -- one 128-bit shared load each in the sweep.  An
// entry whose ring position has bit 2 set keeps its two halves swapped: a
// quarter warp's eight lanes read eight consecutive entries 32 bytes apart,
// and the swap puts their 16-byte halves on distinct banks (without it, two
// lanes of every eight share banks).  Entry e of a chunk therefore has its
// coordinates at byte (e << 5) ^ ((e & 4) << 2) and the rest 16 bytes away.
__device__ __forceinline__ void put_entry(float4 *ring, int pos, float4 xq, float2 prm,
                                          unsigned mask, int jk) {
    const int sw = (pos >> 2) & 1;
    ring[2 * pos + sw] = xq;
    ring[2 * pos + (sw ^ 1)] =
        make_float4(prm.x, prm.y, __uint_as_float(mask), __int_as_float(jk));
}

__device__ __forceinline__ void copy_entry(const float4 *src, int ps, float4 *dst, int pd) {
    const int ss = (ps >> 2) & 1, sd = (pd >> 2) & 1;
    const float4 x = src[2 * ps + ss], au = src[2 * ps + (ss ^ 1)];
    dst[2 * pd + sd] = x;
    dst[2 * pd + (sd ^ 1)] = au;
}

// byte offset of the coordinates half of entry e within its chunk
__device__ __forceinline__ unsigned entry_off(unsigned e) { return (e << 5) ^ ((e & 4u) << 2); }

__device__ __forceinline__ void lds128(unsigned addr, float4 &v) {
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr));
}

// ---- two pairs per instruction -----------------------------------------
// Blackwell's packed FP32 arithmetic (PTX add/mul/fma .f32x2): one
// instruction computes the same operation on two independent (A, B) float
// pairs held in a 64-bit register, each rounded as the scalar instruction
// would.  The whole-warp sweep evaluates this lane's i atom against two j
// atoms per step this way; special functions, compares and selects stay
// scalar on the two halves.
typedef unsigned long long u64;
__device__ __forceinline__ u64 pk2(float a, float b) {
    u64 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpk2(u64 r, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ u64 add2(u64 a, u64 b) {
    u64 r;
    asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
    u64 r;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 mul2(u64 a, u64 b) {
    u64 r;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ u64 fma2(u64 a, u64 b, u64 c) {  // a b + c
    u64 r;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ u64 neg2(u64 a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ u64 splat2(float a) { return pk2(a, a); }
__device__ __forceinline__ u64 lds64(unsigned addr) {
    u64 v;
    asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
    return v;
}

// the Ewald arguments 1 + p beta r and -beta^2 log2(e) r^2 as packed
// operations (1) or on the scalar halves (0: two fewer packed constants)
#ifndef MDG_PK_EWALD_ARGS
#define MDG_PK_EWALD_ARGS 0
#endif

// Packed rings (whole-warp form): a ring of 128 atom slots is two
// super-chunks of 64; a super-chunk is four 512-byte blocks, one per field
// pair -- (x, y), (z, q), (sigma/2, sqrt(4 eps)), (exclusion mask, slot) --
// of 32 16-byte cells.  Atom slot p sits in super-chunk p >> 6, in one half
// of one cell (pk_off), and a cell holds (first field of half A, of half
// B, second field of half A, of half B): one 128-bit load gives a lane both
// fields of one (A, B) pair as two packed operands.  A quarter warp's eight
// lanes read eight cells of one aligned 128-byte run, so the loads are free
// of bank conflicts.
constexpr int kPkRing = 128;   // atom slots per packed ring
constexpr int kPkChunk = 512;  // floats per super-chunk
constexpr int kPkBlock = 128;  // floats per field-pair block
// slot p: half p & 1 of cell (p >> 1) & 31 -- consecutive slots, which a
// warp writes at once, alternate halves, so their 4-byte field writes fall
// on 16 banks (2-way) instead of 8 (4-way)
__device__ __forceinline__ int pk_off(int p) {
    return (p >> 6) * kPkChunk + ((p >> 1) & 31) * 4 + (p & 1);
}
__device__ __forceinline__ float *pk_slot(float *ring, int p) { return ring + pk_off(p); }
__device__ __forceinline__ const float *pk_slot(const float *ring, int p) { return ring + pk_off(p); }
// float offsets of the eight fields of a slot from pk_slot
__device__ __forceinline__ constexpr int pk_field(int f) { return (f >> 1) * kPkBlock + (f & 1) * 2; }
__device__ __forceinline__ void put_entry_pk(float *ring, int p, float4 xq, float2 prm,
                                             unsigned mask, int jk) {
    float *w = pk_slot(ring, p);
    w[pk_field(0)] = xq.x;
    w[pk_field(1)] = xq.y;
    w[pk_field(2)] = xq.z;
    w[pk_field(3)] = xq.w;
    w[pk_field(4)] = prm.x;
    w[pk_field(5)] = prm.y;
    w[pk_field(6)] = __uint_as_float(mask);
    w[pk_field(7)] = __int_as_float(jk);
}
__device__ __forceinline__ void copy_entry_pk(const float *src, int ps, float *dst, int pd) {
    const float *r = pk_slot(src, ps);
    float *w = pk_slot(dst, pd);
#pragma unroll
    for (int f = 0; f < 8; ++f) w[pk_field(f)] = r[pk_field(f)];
}
// one 128-bit shared load: the two packed operands of a field-pair cell
__device__ __forceinline__ void lds2x64(unsigned addr, u64 &a, u64 &b) {
    asm volatile("ld.shared.v2.b64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "r"(addr));
}

// the lane's i atom, replicated into both halves
struct PairI2 {
    u64 X, Y, Z, Q, S, E;
};
// packed constants of the sweep (both halves equal)
struct PkC {
    u64 one, six, twelve, a1, a2, a3, a4, a5, fc, g;
#if MDG_PK_EWALD_ARGS
    u64 bp, negc;
#endif
};

// Two pairs at once: this lane's i atom with the (A, B) j atoms of one
// packed step.  Same arithmetic as pair_interact, each operation applied to
// both pairs, with the CHARMM switch written in the scaled distance
// u = (rc^2 - r^2) / (rc^2 - rs^2), clamped to 1 below rs:
// sw = u^2 (3 - 2u), and -(1/r) d(sw)/dr = 12 u (1 - u) / (rc^2 - rs^2) =: g,
// so the switched LJ force over r is c6 [(12 s^6 - 6) sw / r^2 + (s^6 - 1) g]
// with c6 = 4 eps s^6, s^6 = (sigma / r)^6.  FI accumulates +fr d (the i
// force is its negated sum of the two halves); FJ the two j accumulators;
// n_in (energy variant) counts this lane's pairs inside the cutoff.
template <int COUL, bool LJ, bool SWITCH, bool ENERGY, bool DUMP, bool WL>
__device__ __forceinline__ void pair_interact2(const NbArgs &a, const SysDev &sd,
                                               const PairI2 &I2, const PkC &c, int ik,
                                               unsigned lanebit, u64 X, u64 Y, u64 Z, u64 Qj,
                                               u64 Sj, u64 Ej, u64 M, u64 Jk, u64 &FIX, u64 &FIY,
                                               u64 &FIZ, u64 &FJX, u64 &FJY, u64 &FJZ, u64 &CLJ,
                                               u64 &CC, unsigned &n_in) {
    const u64 DX = sub2(X, I2.X), DY = sub2(Y, I2.Y), DZ = sub2(Z, I2.Z);
    const u64 R2 = fma2(DX, DX, fma2(DY, DY, mul2(DZ, DZ)));
    float r2a, r2b, ma, mb;
    unpk2(R2, r2a, r2b);
    unpk2(M, ma, mb);
    // masked and out-of-range pairs may compute inf/NaN; every use below
    // selects them away
    const bool inca = (r2a <= a.rc2) && !(__float_as_uint(ma) & lanebit);
    const bool incb = (r2b <= a.rc2) && !(__float_as_uint(mb) & lanebit);
    if (DUMP) {
        float ja, jb;
        unpk2(Jk, ja, jb);
        const int pi_atom = a.perm[ik];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (h ? incb : inca) {
                const int pj_atom = a.perm[__float_as_int(h ? jb : ja)];
                if (ref_within32(a.x, pi_atom, pj_atom, sd, a.rc_ref)) {
                    unsigned long long slot = atomicAdd(a.dump_count, 1ull);
                    if ((long long)slot < a.dump_cap) {
                        a.dump[2 * slot] = min(pi_atom, pj_atom);
                        a.dump[2 * slot + 1] = max(pi_atom, pj_atom);
                    }
                }
            }
        }
    }
    const u64 RINV = pk2(rsqrtf(r2a), rsqrtf(r2b));
    const u64 RINV2 = mul2(RINV, RINV);
    u64 FR = 0ull, ELJ = 0ull, ECL = 0ull;
    if (LJ && WL) {
        const u64 SIG = add2(I2.S, Sj);
        const u64 S2 = mul2(mul2(SIG, SIG), RINV2);
        const u64 S6 = mul2(mul2(S2, S2), S2);
        const u64 C6 = mul2(mul2(I2.E, Ej), S6);
        const u64 B = sub2(S6, c.one);           // s^6 - 1
        const u64 A = fma2(B, c.twelve, c.six);  // 12 s^6 - 6
        if (SWITCH) {
            // u on the scalar halves (constants from the arguments)
            const float ua = fminf(fmaf(r2a, a.sw_um, a.sw_uc), 1.0f);
            const float ub = fminf(fmaf(r2b, a.sw_um, a.sw_uc), 1.0f);
            const u64 U = pk2(ua, ub);
            const u64 U2 = mul2(U, U);
            const u64 SW = mul2(U2, pk2(fmaf(-2.0f, ua, 3.0f), fmaf(-2.0f, ub, 3.0f)));
            const u64 G = mul2(sub2(U, U2), c.g);
            FR = mul2(C6, fma2(mul2(A, RINV2), SW, mul2(B, G)));
            if (ENERGY) ELJ = mul2(mul2(C6, B), SW);
        } else {
            FR = mul2(mul2(C6, A), RINV2);
            if (ENERGY) ELJ = mul2(C6, B);
        }
    }
    if (COUL == MDG_COUL_EWALD) {
        const u64 QQ = mul2(I2.Q, Qj);
        const u64 R = mul2(R2, RINV);  // r
        float ta, tb, ea, eb;
#if MDG_PK_EWALD_ARGS
        unpk2(fma2(R, c.bp, c.one), ta, tb);
        unpk2(mul2(R2, c.negc), ea, eb);
#else
        {
            float ra, rb;
            unpk2(R, ra, rb);
            ta = fmaf(a.beta_p, ra, 1.0f);
            tb = fmaf(a.beta_p, rb, 1.0f);
            ea = -a.ewald_exp_c * r2a;
            eb = -a.ewald_exp_c * r2b;
        }
#endif
        const u64 TT = pk2(fast_rcp(ta), fast_rcp(tb));
        const u64 EX = pk2(fast_exp2(ea), fast_exp2(eb));
        const u64 POLY =
            mul2(TT, fma2(TT, fma2(TT, fma2(TT, fma2(TT, c.a5, c.a4), c.a3), c.a2), c.a1));
        // q q e^{-b^2 r^2} (erfc-fit/r + 2 b/sqrt(pi)) / r^2
        FR = fma2(mul2(mul2(QQ, EX), fma2(POLY, RINV, c.fc)), RINV2, FR);
        if (ENERGY) {
            float ua, ub;
            unpk2(TT, ua, ub);
            // q q erfc(beta r) / r = q q t Q(t) e^{-b^2 r^2} / r
            ECL = mul2(mul2(mul2(QQ, TT), pk2(erfc_q(ua), erfc_q(ub))), mul2(EX, RINV));
        }
    }
    float fa, fb;
    unpk2(FR, fa, fb);
    FR = pk2(inca ? fa : 0.f, incb ? fb : 0.f);
    FIX = fma2(FR, DX, FIX);
    FIY = fma2(FR, DY, FIY);
    FIZ = fma2(FR, DZ, FIZ);
    FJX = fma2(FR, DX, FJX);
    FJY = fma2(FR, DY, FJY);
    FJZ = fma2(FR, DZ, FJZ);
    if (ENERGY) {
        float la, lb, ca, cb;
        unpk2(ELJ, la, lb);
        unpk2(ECL, ca, cb);
        CLJ = add2(CLJ, pk2(inca ? la : 0.f, incb ? lb : 0.f));
        CC = add2(CC, pk2(inca ? ca : 0.f, incb ? cb : 0.f));
        n_in += (unsigned)inca + (unsigned)incb;
    }
}

__device__ __forceinline__ u64 shfl_xor2(u64 v, unsigned m) {
    float a, b;
    unpk2(v, a, b);
    return pk2(__shfl_xor_sync(kFull, a, m), __shfl_xor_sync(kFull, b, m));
}

// One pair: this lane's i atom (xi: position and scaled charge; pi: sigma/2
// and sqrt(4 eps); ik its cluster-order slot) with one ring entry (xj:
// shifted position and scaled charge; aux: the entry's sigma/2, sqrt(4 eps),
// exclusion mask of the 32 i lanes and slot).  The force goes to the i
// accumulators (fi) and to the entry's j accumulator (fj), the energies to
// c_lj / c_c (FP32 within a chunk); WL: the entry carries LJ parameters.
template <int COUL, bool LJ, bool SWITCH, bool ENERGY, bool DUMP, bool WL>
__device__ __forceinline__ void pair_interact(const NbArgs &a, const SysDev &sd, const float4 &xi,
                                              const float2 &pi, int ik, unsigned lanebit,
                                              const float4 &xj, const float4 &aux, float &fix,
                                              float &fiy, float &fiz, float &fjx, float &fjy,
                                              float &fjz, float &c_lj, float &c_c,
                                              unsigned long long &n_in) {
    const unsigned mk = __float_as_uint(aux.z);
    const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    // masked and out-of-range pairs may compute inf/NaN (r2 = 0 for an
    // atom with itself); every use below selects them away
    const bool inc = (r2 <= a.rc2) && !(mk & lanebit);
    if (DUMP && inc) {
        // a candidate of the widened search; the reference's own
        // float32 test decides
        const int pj_atom = a.perm[__float_as_int(aux.w)], pi_atom = a.perm[ik];
        if (ref_within32(a.x, pi_atom, pj_atom, sd, a.rc_ref)) {
            unsigned long long slot = atomicAdd(a.dump_count, 1ull);
            if ((long long)slot < a.dump_cap) {
                a.dump[2 * slot] = min(pi_atom, pj_atom);
                a.dump[2 * slot + 1] = max(pi_atom, pj_atom);
            }
        }
    }
    const float rinv = rsqrtf(r2);
    const float rinv2 = rinv * rinv;
    float fr = 0.f, elj = 0.f, ecl = 0.f;
    if (LJ && WL) {
        const float sig = pi.x + aux.x;
        const float s2 = sig * sig * rinv2;
        const float s6 = s2 * s2 * s2;
        const float c6 = pi.y * aux.y * s6;
        float flj = c6 * fmaf(12.0f, s6, -6.0f) * rinv2;
        if (SWITCH) {
            // CHARMM switch, branch free: below rs the clamped r^2 gives
            // sw = 1 and dsw = 0 exactly
            elj = c6 * (s6 - 1.0f);
            const float r2c = fmaxf(r2, a.rs2);
            const float u = a.rc2 - r2c;
            const float sw = u * u * fmaf(2.0f, r2c, a.rc2 - 3.0f * a.rs2) * a.sw_inv_den;
            const float dsw = 12.0f * u * (a.rs2 - r2c) * a.sw_inv_den;
            flj = fmaf(flj, sw, -elj * dsw);
            elj *= sw;
        } else if (ENERGY) {
            elj = c6 * (s6 - 1.0f);
        }
        fr = flj;
    }
    if (COUL == MDG_COUL_EWALD) {
        const float qq = xi.w * xj.w;
        const float r = r2 * rinv;
        const float tt = fast_rcp(fmaf(a.beta_p, r, 1.0f));
        const float poly =
            tt * fmaf(tt, fmaf(tt, fmaf(tt, fmaf(tt, kAsA5, kAsA4), kAsA3), kAsA2), kAsA1);
        const float ex = fast_exp2(-a.ewald_exp_c * r2);
        const float ecf = qq * poly * ex * rinv;
        fr = fmaf(fmaf(qq * a.ewald_fc, ex, ecf), rinv2, fr);
        // the force keeps the 1.5e-7 approximation in every variant (so a
        // trajectory does not depend on when energies are reported); the
        // reported energy uses the relative fit erfc_q, whose error does not
        // pile up over 10^7 pairs
        if (ENERGY) ecl = qq * tt * erfc_q(tt) * ex * rinv;
    }
    fr = inc ? fr : 0.f;
    fix = fmaf(-fr, dx, fix);
    fiy = fmaf(-fr, dy, fiy);
    fiz = fmaf(-fr, dz, fiz);
    fjx = fmaf(fr, dx, fjx);
    fjy = fmaf(fr, dy, fjy);
    fjz = fmaf(fr, dz, fjz);
    if (ENERGY) {
        c_lj += inc ? elj : 0.f;
        c_c += inc ? ecl : 0.f;
        n_in += __popc(__ballot_sync(kFull, inc));
    }
}

// Candidate clusters of i-cluster I for work item `part` (of a.split): every
// (J, periodic image) whose bounding box lies within rc of I's box, offered
// to candidate(J, image code) in ballot order.  Work item `part` scans
// batches part, part + split, ... of 32 clusters, so the split warps of one
// i-cluster share its neighbourhood without talking to each other.
// Balanced half shell: the cluster pair {I, J} (I != J) belongs to I when
// I < J and I + J is odd, or when I > J and I + J is even -- every cluster
// owns about half of its neighbours whatever its index; J == I is kept and
// split by the lane mask.  Periodic images: the nearest image of J's box
// centre, or all 27 when a box pair spans half the box.
template <bool ENERGY, typename Cand>
__device__ __forceinline__ void scan_candidates(const NbArgs &a, const int I, const int part,
                                                const SysDev &sd, const float4 cI,
                                                const float4 hI, Cand &&candidate,
                                                unsigned &n_cand) {
    const float L[3] = {sd.L[0], sd.L[1], sd.L[2]};
    const float invL[3] = {sd.invL[0], sd.invL[1], sd.invL[2]};
    const int cl_lo = sd.cl_off, cl_hi = sd.cl_off + sd.cl_cap;
    const int sid = a.cl_sys[I];
    const int lane = threadIdx.x & 31;
    // every lane offers one (J, image) candidate; the hits go to candidate()
    auto offer = [&](bool hit, int J, int code) {
        unsigned b = __ballot_sync(kFull, hit);
        if (ENERGY) n_cand += __popc(b);
        while (b) {
            const int src = __ffs(b) - 1;
            b &= b - 1;
            candidate(__shfl_sync(kFull, J, src), __shfl_sync(kFull, code, src));
        }
    };
    // the half-shell owner rule
    auto owned = [&](int J) { return J == I || ((I + J) & 1) == (I < J ? 1 : 0); };

    // Column mode (systems whose columns span at least 2R+1 in x and y):
    // candidates come only from the (2R+1)^2 columns around I's column, R =
    // the column reach of rc plus twice the largest distance any cluster box
    // has moved out of its column since the last re-sort.  Each column is a
    // contiguous run of clusters; the runs are concatenated into one virtual
    // list (warp scan of the run lengths) walked 32 at a time.
    int R = 0;
    bool colmode = sd.col_mode != 0;
    if (colmode) {
        const float ov = a.overhang[sid];
        const float aw = fminf(L[0] / (float)sd.ncx, L[1] / (float)sd.ncy);
        R = (int)floorf((a.rc + 2.f * ov) / aw) + 1;
        colmode = 2 * R + 1 <= min(sd.ncx, sd.ncy);
    }
    if (colmode) {
        const int pk = a.col_xy[a.cl_col[I]];
        const int cx = pk >> 16, cy = pk & 0xffff;
        const int side = 2 * R + 1, ncn = side * side;
        const int base0 = a.col_cl_start[sd.col_off];
        for (int cb = 0; cb < ncn; cb += 32) {
            const int c = cb + lane;
            int cnt = 0, start = 0, shc = 4;  // shc: (sx + 1) * 3 + (sy + 1)
            if (c < ncn) {
                int x2 = cx + c / side - R, y2 = cy + c % side - R;
                const int sx = x2 < 0 ? -1 : (x2 >= sd.ncx ? 1 : 0);
                const int sy = y2 < 0 ? -1 : (y2 >= sd.ncy ? 1 : 0);
                x2 -= sx * sd.ncx;
                y2 -= sy * sd.ncy;
                const int gc = sd.col_off + a.col_rank[sd.col_off + x2 * sd.ncy + y2];
                start = sd.cl_off + a.col_cl_start[gc] - base0;
                cnt = a.col_ncl[gc];
                shc = (sx + 1) * 3 + (sy + 1);
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(kFull, incl, 31);
            for (int v0 = part * 32; v0 < total; v0 += a.split * 32) {
                const int v = v0 + lane;
                int lo = 0, hi = 31;  // first lane whose inclusive count exceeds v
#pragma unroll
                for (int it = 0; it < 5; ++it) {
                    const int mid = (lo + hi) >> 1;
                    const int im = __shfl_sync(kFull, incl, mid);
                    if (im > v) hi = mid;
                    else lo = mid + 1;
                }
                const int s_incl = __shfl_sync(kFull, incl, lo);
                const int s_cnt = __shfl_sync(kFull, cnt, lo);
                const int s_start = __shfl_sync(kFull, start, lo);
                const int s_shc = __shfl_sync(kFull, shc, lo);
                const int J = s_start + (v - (s_incl - s_cnt));
                bool valid = v < total && owned(J);
                float4 cJ = make_float4(kFarAway, kFarAway, kFarAway, 0.f),
                       hJ = make_float4(0.f, 0.f, 0.f, 0.f);
                if (valid) {
                    cJ = a.bbox[2 * J];
                    hJ = a.bbox[2 * J + 1];
                }
                valid = valid && cJ.w > 0.f;
                // x and y images follow from the column wrap; z takes the
                // nearest image of the box centres, or all three when a box
                // pair spans half the box height
                const float d[3] = {cJ.x - cI.x, cJ.y - cI.y, cJ.z - cI.z};
                const float h[3] = {hI.x + hJ.x, hI.y + hJ.y, hI.z + hJ.z};
                const float gx = fmaxf(fabsf(fmaf((float)(s_shc / 3 - 1), L[0], d[0])) - h[0], 0.f);
                const float gy = fmaxf(fabsf(fmaf((float)(s_shc % 3 - 1), L[1], d[1])) - h[1], 0.f);
                const float gxy = fmaf(gx, gx, gy * gy);
                float nz = -rintf(d[2] * invL[2]);
                nz = fminf(fmaxf(nz, -1.f), 1.f);
                const float gz = fmaxf(fabsf(fmaf(nz, L[2], d[2])) - h[2], 0.f);
                const bool near_hit = valid && fmaf(gz, gz, gxy) <= a.rc2;
                const bool multi_z = valid && (h[2] + a.rc >= 0.5f * L[2]);
                if (!__any_sync(kFull, multi_z)) {
                    offer(near_hit, J, s_shc * 3 + (int)nz + 1);
                } else {
                    for (int zz = -1; zz <= 1; ++zz) {
                        bool hit = near_hit && zz == (int)nz;
                        if (multi_z) {
                            const float g = fmaxf(fabsf(fmaf((float)zz, L[2], d[2])) - h[2], 0.f);
                            hit = fmaf(g, g, gxy) <= a.rc2;
                        }
                        offer(hit, J, s_shc * 3 + zz + 1);
                    }
                }
            }
        }
    } else {
        // full scan of the system's clusters: work item `part` takes batches
        // part, part + split, ... of 32 clusters
        for (int J0 = cl_lo + part * 32; J0 < cl_hi; J0 += a.split * 32) {
            const int J = J0 + lane;
            bool valid = J < cl_hi && owned(J);
            float4 cJ = make_float4(kFarAway, kFarAway, kFarAway, 0.f),
                   hJ = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                cJ = a.bbox[2 * J];
                hJ = a.bbox[2 * J + 1];
            }
            const float d[3] = {cJ.x - cI.x, cJ.y - cI.y, cJ.z - cI.z};
            const float h[3] = {hI.x + hJ.x, hI.y + hJ.y, hI.z + hJ.z};
            int ncode = 0;
            float g2 = 0.f;
            bool multi = false;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float nk = -rintf(d[k] * invL[k]);
                nk = fminf(fmaxf(nk, -1.f), 1.f);
                const float dd = fmaf(nk, L[k], d[k]);
                const float gap = fmaxf(fabsf(dd) - h[k], 0.f);
                g2 = fmaf(gap, gap, g2);
                ncode = ncode * 3 + (int)nk + 1;
                multi = multi || (h[k] + a.rc >= 0.5f * L[k]);
            }
            valid = valid && cJ.w > 0.f;
            multi = multi && valid;
            const bool near_hit = valid && g2 <= a.rc2;
            if (!__any_sync(kFull, multi)) {
                offer(near_hit, J, ncode);
            } else {
                for (int code = 0; code < 27; ++code) {
                    bool hit = near_hit && code == ncode;
                    if (multi) {
                        const int s3[3] = {code / 9 - 1, (code / 3) % 3 - 1, code % 3 - 1};
                        float gg = 0.f;
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const float dd = fmaf((float)s3[k], L[k], d[k]);
                            const float gap = fmaxf(fabsf(dd) - h[k], 0.f);
                            gg = fmaf(gap, gap, gg);
                        }
                        hit = gg <= a.rc2;
                    }
                    offer(hit, J, code);
                }
            }
        }
    }
}

// One work item: part `part` (of a.split) of i-cluster I's pair search.
// HALF: the warp's two 16-lane halves sweep separate j lists, each holding
// only the j atoms within rc of its own 16 i atoms' box.
template <int COUL, bool LJ, bool SWITCH, bool ENERGY, bool DUMP, bool HALF>
__device__ __forceinline__ void nb_item(const NbArgs &a, const int I, const int part,
                                        float4 *s_j) {
    // rings of 64 entries (2 float4 each): L = j atoms with LJ parameters,
    // Q = charge-only j atoms; in HALF mode one pair of rings per half warp
    float4 *const ringL = s_j, *const ringQ = s_j + 2 * kRing;
    float4 *const ringL2 = s_j + 4 * kRing, *const ringQ2 = s_j + 6 * kRing;
    const float4 cI = a.bbox[2 * I], hI = a.bbox[2 * I + 1];
    if (cI.w == 0.f) return;  // all-padding cluster
    // this cluster's system and its box
    const int sid = a.cl_sys[I];
    const SysDev &sd = a.sys[sid];
    const float L[3] = {sd.L[0], sd.L[1], sd.L[2]};
    const int lane = threadIdx.x;
    const unsigned lt = (1u << lane) - 1u;
    const int ik = I * kCluster + lane;
    const float4 xi = a.xq[ik];
    const float2 pi = a.prm[ik];
    const bool i_real = xi.x < 0.5f * kFarAway;
    const int2 rI = a.prange[I];
    const int ilo = I * kCluster;

    float fix = 0.f, fiy = 0.f, fiz = 0.f;
    double acc_lj = 0.0, acc_c = 0.0;  // per-lane energies: FP32 within a chunk, FP64 across
    // whole warp: the packed rings, this lane's i atom in both halves, the
    // packed constants and the packed i-force sums (+fr d, negated at the end)
    float *const pringL = (float *)s_j, *const pringQ = (float *)s_j + 2 * kPkChunk;
    PairI2 I2;
    I2.X = splat2(xi.x);
    I2.Y = splat2(xi.y);
    I2.Z = splat2(xi.z);
    I2.Q = splat2(xi.w);
    I2.S = splat2(pi.x);
    I2.E = splat2(pi.y);
    PkC pc;
    pc.one = splat2(1.0f);
    pc.six = splat2(6.0f);
    pc.twelve = splat2(12.0f);
    pc.a1 = splat2(kAsA1);
    pc.a2 = splat2(kAsA2);
    pc.a3 = splat2(kAsA3);
    pc.a4 = splat2(kAsA4);
    pc.a5 = splat2(kAsA5);
    pc.fc = splat2(a.ewald_fc);
    pc.g = splat2(a.sw_g);
#if MDG_PK_EWALD_ARGS
    pc.bp = splat2(a.beta_p);
    pc.negc = splat2(-a.ewald_exp_c);
#endif
    unsigned n_in_lane = 0;  // energy variant: this lane's in-cutoff pairs (packed sweep)
    u64 FIX = 0ull, FIY = 0ull, FIZ = 0ull;
    unsigned long long n_eval = 0, n_in = 0;
    // two rings: j atoms with LJ parameters, and charge-only j atoms, whose
    // sweeps skip the LJ arithmetic (two of every three water atoms)
    int jbL = 0, jcL = 0, jbQ = 0, jcQ = 0;
    int jbL2 = 0, jcL2 = 0, jbQ2 = 0, jcQ2 = 0;  // second half warp (HALF mode)

    // Sweep of one 32-entry chunk starting at ring slot `base` (0 or 32).  At
    // step t lane l pairs its i atom with entry l ^ t and keeps the i force;
    // the j-force accumulator of entry e travels so that it always sits in
    // the lane that pairs with e next (a butterfly shuffle with mask
    // t ^ (t + 1)).  After step 31 lane l owns entry l ^ 31's complete j
    // force.  The chunk is 1024-byte aligned, so entry l ^ t lives at
    // chunk | entry_off(l ^ t): one logic op per step for the address.
    const unsigned lanebit = 1u << lane;
    auto chunk = [&](auto with_lj, auto width, unsigned sa) {
        constexpr bool WL = decltype(with_lj)::value;
        constexpr int W = decltype(width)::value;  // 32: whole warp; 16: per half warp
        const int li = lane & (W - 1);
        float fjx = 0.f, fjy = 0.f, fjz = 0.f;
        float c_lj = 0.f, c_c = 0.f;
        auto step = [&](const float4 &xj, const float4 &aux, unsigned shfl_mask) {
            pair_interact<COUL, LJ, SWITCH, ENERGY, DUMP, WL>(a, sd, xi, pi, ik, lanebit, xj, aux,
                                                             fix, fiy, fiz, fjx, fjy, fjz, c_lj,
                                                             c_c, n_in);
            fjx = __shfl_xor_sync(kFull, fjx, shfl_mask);
            fjy = __shfl_xor_sync(kFull, fjy, shfl_mask);
            fjz = __shfl_xor_sync(kFull, fjz, shfl_mask);
        };
        // each step's entry is loaded one step ahead, so its shared-memory
        // latency overlaps the previous step's arithmetic
        float4 xa, aa, xb, ab;
        const unsigned s0 = sa | entry_off((unsigned)li);
        lds128(s0, xa);
        lds128(s0 ^ 16u, aa);
#pragma unroll 1
        for (int t0 = 0; t0 < W; t0 += 4) {
            // entries (l ^ t0) .. (l ^ t0) ^ 3 share bit 2, hence the swap
            const unsigned sb = sa | entry_off((unsigned)(li ^ t0));
            // masks t ^ (t + 1) for t = t0 .. t0 + 3 (below W: a half warp's
            // accumulators stay in that half); none after the last step
            const unsigned m3 = t0 == W - 4 ? 0u : (unsigned)((t0 + 3) ^ (t0 + 4));
            lds128(sb ^ 32u, xb);
            lds128(sb ^ 48u, ab);
            step(xa, aa, 1u);
            lds128(sb ^ 64u, xa);
            lds128(sb ^ 80u, aa);
            step(xb, ab, 3u);
            lds128(sb ^ 96u, xb);
            lds128(sb ^ 112u, ab);
            step(xa, aa, 1u);
            if (t0 < W - 4) {
                const unsigned nb = sa | entry_off((unsigned)(li ^ (t0 + 4)));
                lds128(nb, xa);
                lds128(nb ^ 16u, aa);
            }
            step(xb, ab, m3);
        }
        float4 own;
        lds128((sa | entry_off((unsigned)(li ^ (W - 1)))) ^ 16u, own);
        const int jk = __float_as_int(own.w);
        if (jk >= 0 && !DUMP) {
            if (!(fabsf(fjx) < kFixLimit && fabsf(fjy) < kFixLimit && fabsf(fjz) < kFixLimit))
                raise_status(a.status, MDG_ERR_OVERFLOW);
            fix_red(&a.f[jk], to_fix(fjx));
            fix_red(&a.f[a.n_pad + jk], to_fix(fjy));
            fix_red(&a.f[2 * a.n_pad + jk], to_fix(fjz));
        }
        if (ENERGY) {
            acc_lj += (double)c_lj;
            acc_c += (double)c_c;
        }
        n_eval += W * 32;
        __syncwarp();
    };
    auto shared_addr = [](const float4 *p) { return (unsigned)__cvta_generic_to_shared(p); };
    auto shared_addr_f = [](const float *p) { return (unsigned)__cvta_generic_to_shared(p); };
    auto push_j = [&](int jk, float fjx, float fjy, float fjz) {
        if (jk >= 0 && !DUMP) {
            if (!(fabsf(fjx) < kFixLimit && fabsf(fjy) < kFixLimit && fabsf(fjz) < kFixLimit))
                raise_status(a.status, MDG_ERR_OVERFLOW);
            fix_red(&a.f[jk], to_fix(fjx));
            fix_red(&a.f[a.n_pad + jk], to_fix(fjy));
            fix_red(&a.f[2 * a.n_pad + jk], to_fix(fjz));
        }
    };
    // Whole warp: one packed super-chunk (64 j atoms as 32 (A, B) pairs) at
    // byte address sa, swept in 32 rotation steps: at step t lane l pairs its
    // i atom with pair l ^ t (both halves at once), the pair's j-force
    // accumulators travel by butterfly shuffles (mask t ^ (t + 1)), and
    // after step 31 lane l owns pair l ^ 31's two j forces.  (Loading each
    // step's fields one step ahead was measured slower, 0.244 against 0.237
    // ms on the 88k-atom box.)
    auto chunk64 = [&](auto with_lj, unsigned sa) {
        constexpr bool WL = decltype(with_lj)::value;
        u64 FJX = 0ull, FJY = 0ull, FJZ = 0ull, CLJ = 0ull, CC = 0ull;
        // sa is 2048-byte aligned: cell l ^ t of a block lies at
        // (sa | l << 4) ^ t << 4; the last step needs no shuffle
        const unsigned base = sa | ((unsigned)lane << 4);
        auto step = [&](unsigned t) {
            const unsigned ad = base ^ (t << 4);
            u64 X, Y, Z, Q, S = 0ull, E = 0ull, M, J = 0ull;
            lds2x64(ad, X, Y);
            lds2x64(ad + 512u, Z, Q);
            if (LJ && WL) lds2x64(ad + 1024u, S, E);
            if (DUMP) lds2x64(ad + 1536u, M, J);
            else M = lds64(ad + 1536u);
            pair_interact2<COUL, LJ, SWITCH, ENERGY, DUMP, WL>(a, sd, I2, pc, ik, lanebit, X, Y, Z, Q,
                                                              S, E, M, J, FIX, FIY, FIZ, FJX,
                                                              FJY, FJZ, CLJ, CC, n_in_lane);
        };
#pragma unroll 1
        for (unsigned t = 0; t < 31u; ++t) {
            step(t);
            const unsigned m = t ^ (t + 1u);
            FJX = shfl_xor2(FJX, m);
            FJY = shfl_xor2(FJY, m);
            FJZ = shfl_xor2(FJZ, m);
        }
        step(31u);
        float ja, jb, xa, xb, ya, yb, za, zb;
        unpk2(lds64(sa + ((unsigned)(lane ^ 31) << 4) + 1544u), ja, jb);
        unpk2(FJX, xa, xb);
        unpk2(FJY, ya, yb);
        unpk2(FJZ, za, zb);
        push_j(__float_as_int(ja), xa, ya, za);
        push_j(__float_as_int(jb), xb, yb, zb);
        if (ENERGY) {
            float p0, p1, q0, q1;
            unpk2(CLJ, p0, p1);
            unpk2(CC, q0, q1);
            acc_lj += (double)p0 + (double)p1;
            acc_c += (double)q0 + (double)q1;
        }
        n_eval += 2048;
        __syncwarp();
    };

    // HALF mode: one 16-step sweep of up to 16 entries of each half's ring of
    // one kind; a half with fewer pending entries is padded with far-away ones
    auto sweep16 = [&](auto with_lj) {
        constexpr bool WL = decltype(with_lj)::value;
        int &cA = WL ? jcL : jcQ, &bA = WL ? jbL : jbQ;
        int &cB = WL ? jcL2 : jcQ2, &bB = WL ? jbL2 : jbQ2;
        float4 *const rA = WL ? ringL : ringQ, *const rB = WL ? ringL2 : ringQ2;
        const int h = lane >> 4, li = lane & 15;
        const int c = h ? cB : cA, b = h ? bB : bA;
        float4 *const r = h ? rB : rA;
        if (li >= c)
            put_entry(r, (b + li) & (kRing - 1), make_float4(kFarAway, kFarAway, kFarAway, 0.f),
                      make_float2(0.f, 0.f), kFull, -1);
        __syncwarp();
        chunk(with_lj, std::integral_constant<int, 16>{}, shared_addr(r + 2 * b));
        cA -= min(16, cA);
        bA = (bA + 16) & (kRing - 1);
        cB -= min(16, cB);
        bB = (bB + 16) & (kRing - 1);
    };

    // one candidate (J, image) found by the scan: test J's atoms against I's box
    // and append the survivors to this warp's ring (chunk sweeps when full)
    auto candidate = [&](int J, int code) {
        float sx, sy, sz;
        decode_shift(code, L, sx, sy, sz);
        const int jk = J * kCluster + lane;
        float4 xj = a.xq[jk];
        xj.x += sx;
        xj.y += sy;
        xj.z += sz;
        // exclusion mask of the i lanes for this j atom
        auto excl_mask = [&]() {
            unsigned m = 0u;
            if (J == I) m = kFull << lane;  // half shell inside the cluster
            if (rI.y >= J * kCluster && rI.x < (J + 1) * kCluster) {
                for (int w = 0; w < a.pw; ++w) {
                    const int p = a.partners[(size_t)jk * a.pw + w];
                    if (p >= 0) {
                        const int pk = (p & 0x3fffffff) - ilo;
                        if (pk >= 0 && pk < kCluster) m |= 1u << pk;
                    }
                }
            }
            return m;
        };
        if constexpr (HALF) {
            auto box_hit = [&](const float4 c, const float4 h) {
                const float ux = fmaxf(fabsf(xj.x - c.x) - h.x, 0.f);
                const float uy = fmaxf(fabsf(xj.y - c.y) - h.y, 0.f);
                const float uz = fmaxf(fabsf(xj.z - c.z) - h.z, 0.f);
                return fmaf(ux, ux, fmaf(uy, uy, uz * uz)) <= a.rc2;
            };
            // a half with no atoms has a far-away box, which far-away padding
            // j slots would "hit": its w (1 when the half has atoms) gates it
            const float4 cA = a.hbox[4 * I], cB = a.hbox[4 * I + 2];
            const bool hitA = cA.w > 0.f && box_hit(cA, a.hbox[4 * I + 1]);
            const bool hitB = cB.w > 0.f && box_hit(cB, a.hbox[4 * I + 3]);
            const float2 pj = (hitA || hitB) ? a.prm[jk] : make_float2(0.f, 0.f);
            const bool to_l = !a.split_rings || (LJ && pj.y != 0.f);
            const bool keep_q = COUL == MDG_COUL_EWALD || DUMP;
            const bool aL = hitA && to_l, aQ = hitA && !to_l && keep_q;
            const bool bL = hitB && to_l, bQ = hitB && !to_l && keep_q;
            const unsigned mAL = __ballot_sync(kFull, aL), mAQ = __ballot_sync(kFull, aQ);
            const unsigned mBL = __ballot_sync(kFull, bL), mBQ = __ballot_sync(kFull, bQ);
            if ((mAL | mAQ | mBL | mBQ) == 0u) return;
            if (aL || aQ || bL || bQ) {
                const unsigned m = excl_mask();
                if (aL) put_entry(ringL, (jbL + jcL + __popc(mAL & lt)) & (kRing - 1), xj, pj, m, jk);
                if (aQ) put_entry(ringQ, (jbQ + jcQ + __popc(mAQ & lt)) & (kRing - 1), xj, pj, m, jk);
                if (bL) put_entry(ringL2, (jbL2 + jcL2 + __popc(mBL & lt)) & (kRing - 1), xj, pj, m, jk);
                if (bQ) put_entry(ringQ2, (jbQ2 + jcQ2 + __popc(mBQ & lt)) & (kRing - 1), xj, pj, m, jk);
            }
            jcL += __popc(mAL);
            jcQ += __popc(mAQ);
            jcL2 += __popc(mBL);
            jcQ2 += __popc(mBQ);
            __syncwarp();
            // every ring stays below 32 pending entries between candidates
            while (jcL >= 32 || jcL2 >= 32 || (jcL >= 16 && jcL2 >= 16)) sweep16(std::true_type{});
            while (jcQ >= 32 || jcQ2 >= 32 || (jcQ >= 16 && jcQ2 >= 16)) sweep16(std::false_type{});
            return;
        }
        const float gx = fmaxf(fabsf(xj.x - cI.x) - hI.x, 0.f);
        const float gy = fmaxf(fabsf(xj.y - cI.y) - hI.y, 0.f);
        const float gz = fmaxf(fabsf(xj.z - cI.z) - hI.z, 0.f);
        const bool hit = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) <= a.rc2;
        const float2 pj = hit ? a.prm[jk] : make_float2(0.f, 0.f);
        // With split rings, LJ-carrying atoms go to ring L and the rest,
        // which matter only for the Ewald term (or the pair-set dump), to
        // ring Q; otherwise every hit goes to ring L.
        const bool to_l = !a.split_rings || (LJ && pj.y != 0.f);
        const bool hitL = hit && to_l;
        const bool hitQ = hit && !to_l && (COUL == MDG_COUL_EWALD || DUMP);
        const unsigned bL = __ballot_sync(kFull, hitL), bQ = __ballot_sync(kFull, hitQ);
        if ((bL | bQ) == 0u) return;
        if (hitL || hitQ) {
            const unsigned m = excl_mask();
            if (hitL)
                put_entry_pk(pringL, (jbL + jcL + __popc(bL & lt)) & (kPkRing - 1), xj, pj, m, jk);
            else
                put_entry_pk(pringQ, (jbQ + jcQ + __popc(bQ & lt)) & (kPkRing - 1), xj, pj, m, jk);
        }
        jcL += __popc(bL);
        jcQ += __popc(bQ);
        __syncwarp();
        // a full super-chunk of a ring is swept; between candidates a ring
        // holds fewer than 64 pending slots (a candidate adds at most 32, so
        // never more than 95 of 128)
        if (jcL >= 64) {
            chunk64(std::true_type{}, shared_addr_f(pringL + (jbL >> 6) * kPkChunk));
            jbL = (jbL + 64) & (kPkRing - 1);
            jcL -= 64;
        }
        if (jcQ >= 64) {
            chunk64(std::false_type{}, shared_addr_f(pringQ + (jbQ >> 6) * kPkChunk));
            jbQ = (jbQ + 64) & (kPkRing - 1);
            jcQ -= 64;
        }
    };

    unsigned n_cand = 0;
    scan_candidates<ENERGY>(a, I, part, sd, cI, hI, candidate, n_cand);
    // The partial last chunks, padded with far-away entries.  When both fit
    // in one chunk the charge-only entries join the LJ chunk (their LJ terms
    // are zero), so an item ends with at most one partial sweep.
    if constexpr (HALF) {
        if ((jcQ > 0 || jcQ2 > 0) && jcL + jcQ <= 16 && jcL2 + jcQ2 <= 16) {
            const int h = lane >> 4, li = lane & 15;
            const int cq = h ? jcQ2 : jcQ;
            if (li < cq)
                copy_entry(h ? ringQ2 : ringQ, ((h ? jbQ2 : jbQ) + li) & (kRing - 1),
                           h ? ringL2 : ringL,
                           ((h ? jbL2 : jbL) + (h ? jcL2 : jcL) + li) & (kRing - 1));
            jcL += jcQ;
            jcQ = 0;
            jcL2 += jcQ2;
            jcQ2 = 0;
            __syncwarp();
        }
        while (jcL > 0 || jcL2 > 0) sweep16(std::true_type{});
        while (jcQ > 0 || jcQ2 > 0) sweep16(std::false_type{});
    }
    if constexpr (!HALF) {
        // the partial super-chunks: charge-only slots join the LJ ring when
        // both fit in one (their LJ terms are zero), then each partial one is
        // padded with far-away slots up to 64 and swept
        if (jcQ > 0 && jcL + jcQ <= 64) {
            for (int k = lane; k < jcQ; k += 32)
                copy_entry_pk(pringQ, (jbQ + k) & (kPkRing - 1), pringL,
                              (jbL + jcL + k) & (kPkRing - 1));
            jcL += jcQ;
            jcQ = 0;
            __syncwarp();
        }
        auto finish = [&](auto with_lj, float *ring, int jb, int jc) {
            if (jc == 0) return;
            for (int k = jc + lane; k < 64; k += 32)
                put_entry_pk(ring, (jb + k) & (kPkRing - 1),
                             make_float4(kFarAway, kFarAway, kFarAway, 0.f), make_float2(0.f, 0.f),
                             kFull, -1);
            __syncwarp();
            chunk64(with_lj, shared_addr_f(ring + (jb >> 6) * kPkChunk));
        };
        finish(std::true_type{}, pringL, jbL, jcL);
        finish(std::false_type{}, pringQ, jbQ, jcQ);
        float a0, a1, b0, b1, c0, c1;
        unpk2(FIX, a0, a1);
        unpk2(FIY, b0, b1);
        unpk2(FIZ, c0, c1);
        fix -= a0 + a1;
        fiy -= b0 + b1;
        fiz -= c0 + c1;
        if (ENERGY) n_in += __reduce_add_sync(kFull, n_in_lane);
    }

    // ---- this work item's share of the i forces and energies -------------
    if (!DUMP && i_real) {
        if (!(fabsf(fix) < kFixLimit && fabsf(fiy) < kFixLimit && fabsf(fiz) < kFixLimit))
            raise_status(a.status, MDG_ERR_OVERFLOW);
        fix_red(&a.f[ik], to_fix(fix));
        fix_red(&a.f[a.n_pad + ik], to_fix(fiy));
        fix_red(&a.f[2 * a.n_pad + ik], to_fix(fiz));
    }
    if (ENERGY) {
        const double el = warp_sum_d(acc_lj), ee = warp_sum_d(acc_c);
        if (lane == 0) {
            if (!(fabs(el) < kFixLimit && fabs(ee) < kFixLimit))
                raise_status(a.status, MDG_ERR_OVERFLOW);
            long long *es = a.energy + sid * kEnergySlots;
            fix_red((unsigned long long *)&es[MDG_TERM_LJ], to_fix_d(el));
            fix_red((unsigned long long *)&es[MDG_TERM_COUL_REAL], to_fix_d(ee));
            atomicAdd(&a.stats[0], n_eval);
            atomicAdd(&a.stats[1], n_in);
            atomicAdd(&a.stats[2], (unsigned long long)n_cand);
            if (part == 0) atomicAdd(&a.stats[3], 1ull);
        }
    }
}

// One work item of the quarter form: the warp's four 8-lane groups hold the
// four 8-slot quarters of i-cluster I, and each group sweeps its own j lists
// -- the j atoms within rc of its quarter's box, fewer than within rc of the
// whole cluster's box.  Each group keeps two rings of 64 entries (LJ-
// carrying and charge-only j atoms); a candidate cluster's atoms are tested
// against the four quarter boxes (kept in shared memory) and appended to
// the rings of the quarters they reach.  A sweep takes one 8-entry chunk
// per group in 8 steps: lane (g, l) pairs its i atom with entry l ^ t of
// its group's chunk, the j-force accumulators move by butterfly shuffles
// inside the group, and after step 7 the lane owns entry l ^ 7's j force.
// A group short of a chunk is padded with far-away entries only when
// another group's ring nears capacity, and at the end of the item.
template <int COUL, bool LJ, bool SWITCH, bool ENERGY, bool DUMP>
__device__ __forceinline__ void nb_item_q(const NbArgs &a, const int I, const int part,
                                          float4 *s_j) {
    constexpr int RQ = 64;  // entries per ring
    // ring (group g, kind k: 0 = LJ, 1 = charge-only) at s_j + (2 g + k) 2 RQ;
    // the four quarter boxes behind the eight rings
    float4 *const qb = s_j + 16 * RQ;
    const float4 cI = a.bbox[2 * I], hI = a.bbox[2 * I + 1];
    if (cI.w == 0.f) return;  // all-padding cluster
    const int sid = a.cl_sys[I];
    const SysDev &sd = a.sys[sid];
    const float L[3] = {sd.L[0], sd.L[1], sd.L[2]};
    const int lane = threadIdx.x;
    const int grp = lane >> 3, li = lane & 7;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned lanebit = 1u << lane;
    const int ik = I * kCluster + lane;
    const float4 xi = a.xq[ik];
    const float2 pi = a.prm[ik];
    const bool i_real = xi.x < 0.5f * kFarAway;
    const int2 rI = a.prange[I];
    const int ilo = I * kCluster;
    __syncwarp();  // a previous item's reads of the boxes are done
    if (lane < 8) qb[lane] = a.qbox[8 * I + lane];
    __syncwarp();
    auto ring = [&](int g, int k) { return s_j + (2 * g + k) * 2 * RQ; };
    auto shared_addr = [](const float4 *p) { return (unsigned)__cvta_generic_to_shared(p); };

    float fix = 0.f, fiy = 0.f, fiz = 0.f;
    double acc_lj = 0.0, acc_c = 0.0;
    unsigned long long n_eval = 0, n_in = 0;
    // this lane's group's rings: first pending entry and pending count
    int jbL = 0, jcL = 0, jbQ = 0, jcQ = 0;

    auto push_j = [&](int jk, float fjx, float fjy, float fjz) {
        if (jk >= 0 && !DUMP) {
            if (!(fabsf(fjx) < kFixLimit && fabsf(fjy) < kFixLimit && fabsf(fjz) < kFixLimit))
                raise_status(a.status, MDG_ERR_OVERFLOW);
            fix_red(&a.f[jk], to_fix(fjx));
            fix_red(&a.f[a.n_pad + jk], to_fix(fjy));
            fix_red(&a.f[2 * a.n_pad + jk], to_fix(fjz));
        }
    };
    // a group short of a chunk of kind k gets far-away entries up to 8
    auto pad = [&](int k, int jb, int jc) {
        if (li >= jc)
            put_entry(ring(grp, k), (jb + li) & (RQ - 1),
                      make_float4(kFarAway, kFarAway, kFarAway, 0.f), make_float2(0.f, 0.f), kFull,
                      -1);
    };
    // One 8-step sweep of one chunk per group (kind k of each group's ring),
    // each step's entry loaded one step ahead; the chunk is 256-byte aligned,
    // so entry l ^ t lives at chunk | entry_off(l ^ t).
    auto sweep = [&](auto with_lj, int k, int jb) {
        constexpr bool WL = decltype(with_lj)::value;
        const unsigned sa = shared_addr(ring(grp, k) + 2 * jb);
        auto at = [&](int t) { return sa | entry_off((unsigned)(li ^ t)); };
        float fx = 0.f, fy = 0.f, fz = 0.f, c_lj = 0.f, c_c = 0.f;
        float4 xa, aa, xb, ab;
        lds128(at(0), xa);
        lds128(at(0) ^ 16u, aa);
#pragma unroll 1
        for (int t = 0; t < 8; t += 2) {
            const unsigned o1 = at(t + 1);
            lds128(o1, xb);
            lds128(o1 ^ 16u, ab);
            pair_interact<COUL, LJ, SWITCH, ENERGY, DUMP, WL>(a, sd, xi, pi, ik, lanebit, xa, aa,
                                                             fix, fiy, fiz, fx, fy, fz, c_lj, c_c,
                                                             n_in);
            fx = __shfl_xor_sync(kFull, fx, 1);
            fy = __shfl_xor_sync(kFull, fy, 1);
            fz = __shfl_xor_sync(kFull, fz, 1);
            if (t < 6) {
                const unsigned o2 = at(t + 2);
                lds128(o2, xa);
                lds128(o2 ^ 16u, aa);
            }
            pair_interact<COUL, LJ, SWITCH, ENERGY, DUMP, WL>(a, sd, xi, pi, ik, lanebit, xb, ab,
                                                             fix, fiy, fiz, fx, fy, fz, c_lj, c_c,
                                                             n_in);
            const int m = t < 6 ? ((t + 1) ^ (t + 2)) : 0;
            fx = __shfl_xor_sync(kFull, fx, m);
            fy = __shfl_xor_sync(kFull, fy, m);
            fz = __shfl_xor_sync(kFull, fz, m);
        }
        float4 own;
        lds128(at(7) ^ 16u, own);
        push_j(__float_as_int(own.w), fx, fy, fz);
        if (ENERGY) {
            acc_lj += (double)c_lj;
            acc_c += (double)c_c;
        }
        n_eval += 256;
        __syncwarp();
    };
    auto take = [](int &jb, int &jc) {
        jb = (jb + 8) & (RQ - 1);
        jc = max(jc - 8, 0);
    };
    // Sweeps after a candidate: a kind whose rings all hold a full chunk;
    // then, while some group's ring could not take another candidate (more
    // than 32 pending), padded sweeps of that kind.  At the end (final_)
    // everything left is swept, padded.
    auto drain = [&](bool final_) {
        const int lim = final_ ? 0 : 32;
        for (;;) {
            if (__all_sync(kFull, jcL >= 8)) {
                sweep(std::true_type{}, 0, jbL);
                take(jbL, jcL);
            } else if (__all_sync(kFull, jcQ >= 8)) {
                sweep(std::false_type{}, 1, jbQ);
                take(jbQ, jcQ);
            } else if (__any_sync(kFull, jcQ > lim)) {
                pad(1, jbQ, jcQ);
                __syncwarp();
                sweep(std::false_type{}, 1, jbQ);
                take(jbQ, jcQ);
            } else if (__any_sync(kFull, jcL > lim)) {
                pad(0, jbL, jcL);
                __syncwarp();
                sweep(std::true_type{}, 0, jbL);
                take(jbL, jcL);
            } else {
                break;
            }
        }
    };

    auto candidate = [&](int J, int code) {
        float sx, sy, sz;
        decode_shift(code, L, sx, sy, sz);
        const int jk = J * kCluster + lane;
        float4 xj = a.xq[jk];
        xj.x += sx;
        xj.y += sy;
        xj.z += sz;
        unsigned hm = 0u;  // the quarters this j atom reaches
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const float4 c = qb[2 * g], h = qb[2 * g + 1];
            const float gx = fmaxf(fabsf(xj.x - c.x) - h.x, 0.f);
            const float gy = fmaxf(fabsf(xj.y - c.y) - h.y, 0.f);
            const float gz = fmaxf(fabsf(xj.z - c.z) - h.z, 0.f);
            // a quarter with no atoms has a far-away box (w = 0), which
            // far-away padding j slots would reach
            if (c.w > 0.f && fmaf(gx, gx, fmaf(gy, gy, gz * gz)) <= a.rc2) hm |= 1u << g;
        }
        const float2 pj = hm ? a.prm[jk] : make_float2(0.f, 0.f);
        const bool to_l = !a.split_rings || (LJ && pj.y != 0.f);
        if (!to_l && !(COUL == MDG_COUL_EWALD || DUMP)) hm = 0u;
        if (__ballot_sync(kFull, hm != 0u) == 0u) return;
        unsigned m = 0u;  // exclusion mask of the 32 i lanes for this j atom
        if (hm) {
            if (J == I) m = kFull << lane;  // half shell inside the cluster
            if (rI.y >= J * kCluster && rI.x < (J + 1) * kCluster) {
                for (int w = 0; w < a.pw; ++w) {
                    const int p = a.partners[(size_t)jk * a.pw + w];
                    if (p >= 0) {
                        const int pk = (p & 0x3fffffff) - ilo;
                        if (pk >= 0 && pk < kCluster) m |= 1u << pk;
                    }
                }
            }
        }
        const int endL = jbL + jcL, endQ = jbQ + jcQ;  // this lane's group's ring ends
        int addL = 0, addQ = 0;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const bool hit = (hm >> g) & 1u;
            const unsigned bL = __ballot_sync(kFull, hit && to_l);
            const unsigned bQ = __ballot_sync(kFull, hit && !to_l);
            const int eL = __shfl_sync(kFull, endL, 8 * g), eQ = __shfl_sync(kFull, endQ, 8 * g);
            if (hit) {
                if (to_l) put_entry(ring(g, 0), (eL + __popc(bL & lt)) & (RQ - 1), xj, pj, m, jk);
                else put_entry(ring(g, 1), (eQ + __popc(bQ & lt)) & (RQ - 1), xj, pj, m, jk);
            }
            if (g == grp) {
                addL = __popc(bL);
                addQ = __popc(bQ);
            }
        }
        jcL += addL;
        jcQ += addQ;
        __syncwarp();
        drain(false);
    };

    unsigned n_cand = 0;
    scan_candidates<ENERGY>(a, I, part, sd, cI, hI, candidate, n_cand);
    drain(true);

    if (!DUMP && i_real) {
        if (!(fabsf(fix) < kFixLimit && fabsf(fiy) < kFixLimit && fabsf(fiz) < kFixLimit))
            raise_status(a.status, MDG_ERR_OVERFLOW);
        fix_red(&a.f[ik], to_fix(fix));
        fix_red(&a.f[a.n_pad + ik], to_fix(fiy));
        fix_red(&a.f[2 * a.n_pad + ik], to_fix(fiz));
    }
    if (ENERGY) {
        const double el = warp_sum_d(acc_lj), ee = warp_sum_d(acc_c);
        if (lane == 0) {
            if (!(fabs(el) < kFixLimit && fabs(ee) < kFixLimit))
                raise_status(a.status, MDG_ERR_OVERFLOW);
            long long *es = a.energy + sid * kEnergySlots;
            fix_red((unsigned long long *)&es[MDG_TERM_LJ], to_fix_d(el));
            fix_red((unsigned long long *)&es[MDG_TERM_COUL_REAL], to_fix_d(ee));
            atomicAdd(&a.stats[0], n_eval);
            atomicAdd(&a.stats[1], n_in);
            atomicAdd(&a.stats[2], (unsigned long long)n_cand);
            if (part == 0) atomicAdd(&a.stats[3], 1ull);
        }
    }
}

// The quarter form as a kernel, in the grid form or the persistent form as
// k_nonbonded below.  16 KB of rings per one-warp CTA: 13 CTAs per SM.
template <int COUL, bool LJ, bool SWITCH, bool ENERGY, bool DUMP>
__global__ void __launch_bounds__(32, ENERGY ? 12 : 13) k_nonbonded_q(NbArgs a) {
    // eight rings of 64 entries of 32 bytes, each 8-entry chunk on a
    // 256-byte boundary, then the four quarter boxes
    __shared__ __align__(1024) float4 s_j[16 * 64 + 8];
    if (!a.persistent) {
        nb_item_q<COUL, LJ, SWITCH, ENERGY, DUMP>(a, blockIdx.x / a.split, blockIdx.x % a.split,
                                                  s_j);
        return;
    }
    for (;;) {
        int base = 0;
        if (threadIdx.x == 0) base = atomicAdd(a.queue, a.grab);
        base = __shfl_sync(kFull, base, 0);
        if (base >= a.n_items) break;
        const int end = min(base + a.grab, a.n_items);
        for (int item = base; item < end; ++item) {
            __syncwarp();
            nb_item_q<COUL, LJ, SWITCH, ENERGY, DUMP>(a, item / a.split, item % a.split, s_j);
        }
    }
}

// Grid form: one one-warp CTA per work item, scheduled by the hardware.
// Persistent form: enough warps to fill the GPU once, each pulling work
// items from a device counter until none is left.
// resident one-warp CTAs per SM the register budget is sized for (96
// registers at 20; the half-warp form's energy variants 128 at 16)
#ifndef MDG_NB_MIN_BLOCKS
#define MDG_NB_MIN_BLOCKS 20
#endif
// the energy variants (an energy step every log interval and at the start)
#ifndef MDG_NB_MIN_BLOCKS_ENERGY
#define MDG_NB_MIN_BLOCKS_ENERGY 20
#endif
#ifndef MDG_NB_CARVEOUT
#define MDG_NB_CARVEOUT 0
#endif
#ifndef MDG_NB_MIN_BLOCKS_HALF
#define MDG_NB_MIN_BLOCKS_HALF 20
#endif
template <int COUL, bool LJ, bool SWITCH, bool ENERGY, bool DUMP, bool HALF>
__global__ void __launch_bounds__(32, ENERGY ? (HALF ? 16 : MDG_NB_MIN_BLOCKS_ENERGY)
                                             : (HALF ? MDG_NB_MIN_BLOCKS_HALF : MDG_NB_MIN_BLOCKS))
    k_nonbonded(NbArgs a) {
    // 8 KB of rings: whole warp, two packed rings of 128 atom slots (two
    // 2 KB super-chunks each); half warp, four rings of 64 entries of 32
    // bytes, each 32-entry chunk on a 1024-byte boundary
    __shared__ __align__(1024) float4 s_j[8 * kRing];
    if (!a.persistent) {
        nb_item<COUL, LJ, SWITCH, ENERGY, DUMP, HALF>(a, blockIdx.x / a.split, blockIdx.x % a.split,
                                                s_j);
        return;
    }
    for (;;) {
        int base = 0;
        if (threadIdx.x == 0) base = atomicAdd(a.queue, a.grab);
        base = __shfl_sync(kFull, base, 0);
        if (base >= a.n_items) break;
        const int end = min(base + a.grab, a.n_items);
        for (int item = base; item < end; ++item) {
            __syncwarp();  // the previous item's ring reads are done
            nb_item<COUL, LJ, SWITCH, ENERGY, DUMP, HALF>(a, item / a.split, item % a.split, s_j);
        }
    }
}

template <int COUL, bool LJ, bool SW, bool HALF>
cudaError_t dispatch_nb(mdg_system *s, const NbArgs &a, int energy, int dump) {
    dim3 grid(a.persistent ? s->nb_persistent_ctas : a.n_items), block(32);
    if (a.persistent && cudaMemsetAsync(a.queue, 0, sizeof(int), s->stream) != cudaSuccess)
        return cudaGetLastError();
    if (dump) {
        if constexpr (COUL == MDG_COUL_EWALD && LJ && !SW)
            k_nonbonded<COUL, LJ, SW, false, true, HALF><<<grid, block, 0, s->stream>>>(a);
    } else if (energy)
        k_nonbonded<COUL, LJ, SW, true, false, HALF><<<grid, block, 0, s->stream>>>(a);
    else {
#if MDG_NB_CARVEOUT
        // the shared-memory carveout at its maximum, so that shared memory
        // does not cap the resident CTAs below the register budget's count
        static bool carveout_set = false;
        if (!carveout_set) {
            cudaFuncSetAttribute(k_nonbonded<COUL, LJ, SW, false, false, HALF>,
                                 cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
            carveout_set = true;
        }
#endif
        k_nonbonded<COUL, LJ, SW, false, false, HALF><<<grid, block, 0, s->stream>>>(a);
    }
    return cudaGetLastError();
}

// every (Coulomb, LJ, switch) combination the library launches, for one HALF
template <bool HALF>
cudaError_t dispatch_shape(mdg_system *s, const NbArgs &a, int coul_tile, bool want_lj, bool sw,
                           int energy, int dump) {
    // the pair-set dump decides pairs by the reference's test alone, whatever
    // the terms: one instantiation serves every configuration
    if (dump) return dispatch_nb<MDG_COUL_EWALD, true, false, HALF>(s, a, 0, 1);
    if (coul_tile == MDG_COUL_EWALD && !want_lj)
        return dispatch_nb<MDG_COUL_EWALD, false, false, HALF>(s, a, energy, dump);
    if (coul_tile == MDG_COUL_EWALD)
        return sw ? dispatch_nb<MDG_COUL_EWALD, true, true, HALF>(s, a, energy, dump)
                  : dispatch_nb<MDG_COUL_EWALD, true, false, HALF>(s, a, energy, dump);
    return sw ? dispatch_nb<MDG_COUL_NONE, true, true, HALF>(s, a, energy, dump)
              : dispatch_nb<MDG_COUL_NONE, true, false, HALF>(s, a, energy, dump);
}

}  // namespace
}  // namespace mdg
