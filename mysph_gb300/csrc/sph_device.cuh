// sph_device.cuh — device-side data layout and per-particle physics shared by
// the hash, pair-pass and integration kernels of libsphgpu.
//
// Layout in HBM (one context):
//   combined particle arrays of N = n_real + n_wall entries; entries
//   [0, n_real) are the real particles in cell-sorted order (re-sorted each
//   step), entries [n_real, N) the static wall particles, sorted by cell once.
//   State that moves with a particle is double-buffered (cur/nxt) so the
//   per-step reorder is one gather:
//     xm  double4 (x, y, z, mass)          vr  double4 (vx, vy, vz, rho)
//     eh  double4 (e, h, c, mass/rho)      dsp double4 (displacement, -)
//     meta int4   (type, boundary, id, state)   id = uploaded index
//     shear double[N*D2] (solid contexts)
//   Per-step arrays in the current order:
//     posf float4 (x-lo, y-lo, z-lo) in FP32 for the candidate filter
//     pa4  double4 (p/rho^2, p, div_v, div_x)
//     tt   double[N*D2]  eta*edot/rho^2 (the viscous term of internal_force)
//     sig  double[N*D2]  stress/rho^2 (solid contexts)
//     ras  double4 (R11, R22, R12, -) artificial-stress tensor (2-D solids)
//     dvr  double4 (dv/dt, drho/dt)  dedt double   dsdt double[N*D2]
//     prev_vr, prev_e, shear_prev: leap-frog "Prev" arrays
//   FP32 mirrors of the mixed-precision pair passes (SPH_PREC_MIXED):
//     pr4 float4 (x, y, z relative to the particle's cell origin, cell code)
//     vf4 float4 (v, rho)   ef4 float4 (h, c, m/rho, m)
//     pf4 float4 (p/rho^2, p, Type bits, -)   tf/sf float[N*D2]   rf4 float4
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sph_gpu.h"
#include "sph_df64.cuh"

#define SPH_FULL_MASK 0xffffffffu

namespace sph {

constexpr int kMaxDim = 3;
constexpr int kMaxD2 = 9;

// status bits written by kernels (ctx->d_status)
constexpr uint32_t ST_NONFINITE = 1u << 0;
constexpr uint32_t ST_RANGE = 1u << 1;    // particle clamped into the border cells
constexpr uint32_t ST_H_RANGE = 1u << 2;  // an evolved smoothing length outgrew its cell size
constexpr uint32_t ST_OVERFLOW = 1u << 2; // neighbour export buffer too small

struct DevMaterial {
    int32_t type, eos, solid, yield;
    double rho0, c0, gamma, K, eta, sigma_y, mg_cs, mg_s;
    double tait_b;   // c0^2 rho0 / gamma
    double inv_rho0, k_rho0;   // 1 / rho0 and K / rho0 (divisions done once, on the host)
    // FP32 copies for the mixed passes (rounded on the host, as a conversion
    // on the device would round them)
    float rho0_f, gamma_f, eta_f, tait_b_f, k_rho0_f, mg_cs_f, mg_s_f;
};

struct Grid {
    double lo[3];
    double inv_cs;      // 1 / cell size
    double cs;
    int nc[3];          // cells per axis (1 on unused axes)
    int ncells;
    float guard;        // relative guard band of the FP32 distance filter (on r^2)
    float cs_f;         // cs in FP32
    // n / nc[a] = (n * div_m[a]) >> (31 + div_l[a]) for 0 <= n < 2^31
    // (a = 0, 1): the multiply-shift reciprocal of Granlund and Montgomery,
    // div_l = ceil(log2 nc), div_m = ceil(2^(31 + div_l) / nc)
    unsigned long long div_m[2];
    int div_l[2];
};

// Cell of a real particle from its sorted cell key (the system's first cell
// plus (c2 nc1 + c1) nc0 + c0), with integer multiplies and shifts: the same
// cell as cell_of on its position, without cell_of's FP64 arithmetic.
__device__ __forceinline__ void cell_from_key(const Grid& g, int base, uint32_t key, int* c) {
    const uint32_t local = key - (uint32_t)base;
    const uint32_t row = (uint32_t)(((unsigned long long)local * g.div_m[0]) >> (31 + g.div_l[0]));
    c[0] = (int)(local - row * (uint32_t)g.nc[0]);
    const uint32_t z = (uint32_t)(((unsigned long long)row * g.div_m[1]) >> (31 + g.div_l[1]));
    c[1] = (int)(row - z * (uint32_t)g.nc[1]);
    c[2] = (int)z;
}

// One particle system of a context.  A plain context holds one instance; a
// batch holds many, each with its own grid (cells [cell_base, cell_base +
// grid.ncells) of the shared cell arrays), material rows, time step and step
// counter, so one launch per stage advances all of them.
struct Inst {
    Grid grid;
    int cell_base;
    int mat_base, n_mat;
    int n_real;        // live real particles (Courant mean)
    int step;          // leap-frog steps taken (device-updated)
    int active;
    int wall_first, n_wall;  // the instance's wall slots [wall_first, +n_wall)
    double dt;
    double time;       // simulated time (device-updated)
    // lengths tied to the particle spacing of each system
    double wall_r0;        // wall-repulsion radius (externalForce.f90:62-101)
    double contact_delta;  // fluid-solid contact distance
    double as_dp;          // artificial-stress reference spacing (artificialTerm.f90:27-32)
    float ext_wall_r2;     // (1.0001 wall_r0)^2: beyond it no wall repulsion
    float ext_delta;       // contact_delta in FP32 (pre-filter of the contact force)
    float wall_r0_f;       // wall_r0 in FP32 (external pair terms of the mixed passes)
};

// Row stride of the FP32 tensor mirrors (tf, sf): Dim^2 floats, padded to 12
// in 3-D so that a row is three aligned float4 loads (a 2-D row is one).
__host__ __device__ constexpr int tf_stride_of(int dim) { return dim == 3 ? 12 : dim * dim; }

struct KRef;

// Device view of a context, passed by value to every kernel.
struct Dev {
    int dim, d2;
    int tfs;          // row stride (floats) of the FP32 tensor mirrors tf / sf
    int n_real, n_wall, n;
    int skf, pa_sph, sle;
    uint32_t flags;
    int scale_k;
    double gravity;
    double av_alpha, av_beta, av_psi, av_alpha_solid, av_beta_solid;
    double av_psi_q, av_alpha_h, av_alpha_h_solid;   // psi^2 / 4, -alpha / 2 (fluid, solid)
    double cour_alpha, cour_beta;
    double wall_fs, wall_p1, wall_p2;
    double pen_factor, pen_n1, pen_n2;
    // FP32 copies for the external pair terms of the mixed passes
    float wall_fs_f, wall_p1_f, wall_p2_f, pen_factor_f, pen_n1_f, pen_n2_f;
    // and for their AV, XSPH (2 eps) and artificial-stress constants
    float av_alpha_f, av_beta_f, av_psi_f, av_alpha_solid_f, av_beta_solid_f, xsph_eps2_f, as_eps_f, as_n_f;
    double as_eps, as_n, xsph_eps;
    const DevMaterial* mat;   // material rows of all instances (global memory)
    Inst* inst;               // instance table (global memory)
    const KRef* kref;         // per instance: kernel constants of its reference h
    int n_inst;
    int total_cells;          // cells of all instances; key of inactive particles
    int wall_off;             // index of the first wall particle
    int has_solid;

    // double-buffered state (cur)
    double4 *xm, *vr, *eh, *dsp;
    int4* meta;
    int* pinst;         // instance of each particle
    double* shear;
    // the other buffer (nxt)
    double4 *xm2, *vr2, *eh2, *dsp2;
    int4* meta2;
    int* pinst2;
    double* shear2;

    float4* posf;
    int precision;     // SPH_PREC_FP64 or SPH_PREC_MIXED
    int tile_k;        // list length per lane of the tiled (mixed) passes
    int tile_tpb;      // threads per block of the tiled (mixed) passes
    int persistent;    // 1: the tiled passes launch only the resident blocks, which stride over the tiles
    int lane_shift;    // log2 of the lanes per target of the FP64 passes A and B (0: one lane)
    float4 *pr4, *vf4, *ef4, *pf4, *rf4;
    float *tf, *sf;
    // double-float mirrors of the DF64 passes (hi in *0, lo in *1):
    // pd = (x, y, z relative to the grid origin, mass), vd = (v, rho),
    // ed0 = (m/rho hi, lo, h hi, lo), ed1 = (c hi, lo, p/rho^2 hi, lo),
    // ttd = eta edot / rho^2 (Dim^2 pairs)
    float4 *pd0, *pd1, *vd0, *vd1, *ed0, *ed1;
    float2* ttd;
    double4* pa4;
    double* tt;
    double* sig;
    double4* ras;
    double4* dvr;
    double* dedt;
    double* dsdt;
    // second buffers of the rates: a reorder without a half kick (sph_nnps,
    // dropping removed systems) carries the last step's rates along
    double4* dvr2;
    double* dedt2;
    double* dsdt2;
    double* tds;
    double* strain;   // edot (parity export)
    double4* prev_vr;
    double* prev_e;
    double* shear_prev;
    double4* aver;    // XSPH correction
    // summation density: the new densities of the real particles, and
    // divergencePosition of the previous step carried through the reorders
    // (double-buffered like the state) for the normalisation test
    double* rsum;
    double* dxp;
    double* dxp2;
    // kernel gradient correction: per real particle the factors of its A_i
    // (KGC_STRIDE doubles, KgcLayout)
    double* kgc;
    // SPH = 3: the walls' uploaded (pressure, sound speed), which the Riemann
    // density of an instance's first step reads (the walls' EOS is applied
    // once at upload; the reference applies it in the first internal_force)
    double2* wraw;
    // SPH = 3: the pressure of the previous EOS in the current particle
    // order (pa4 is rewritten by pass A each step and not carried through
    // the reorder; the permute copies its pressure here)
    double* pold;

    // hash
    uint32_t* keys;       // n_real
    uint32_t* vals;
    uint32_t* keys_s;     // sorted
    uint32_t* vals_s;
    int* fstart;          // ncells + 1 (real particles)
    int* wstart;          // ncells + 1 (walls, offsets into [0, n_wall))
    int* ccount;          // ncells + 1 scratch

    // reductions / status
    unsigned long long* cmax;  // per instance: running max of the Courant number (bits)
    // the Courant sum in a fixed order: per update block its partial sum and
    // instance (-2: the block holds several instances, whose particles'
    // numbers are in cnp)
    double* cpart;
    int* cpinst;
    double* cnp;
    double* cres;              // per instance: [max, mean (carried), sum] of the last step
    uint32_t* status;
    int* nneigh;          // per-particle neighbour counts (statistics/export)
};

__host__ __device__ inline int scale_k_of(int skf) { return skf == 1 ? 2 : ((skf == 2 || skf == 3) ? 3 : 1); }

__device__ __forceinline__ const Inst& inst_of(const Dev& d, int s) { return d.inst[d.pinst[s]]; }

// Slot s belongs to instance f.  Walls are matched by their slot range: the
// walls of a removed instance keep its old id until the batch compacts.
__device__ __forceinline__ bool slot_in_inst(const Dev& d, int s, int f) {
    if (s < d.n_real) return d.pinst[s] == f;
    const Inst& I = d.inst[f];
    return s >= I.wall_first && s < I.wall_first + I.n_wall;
}

__device__ __forceinline__ const DevMaterial* material_of(const Dev& d, const Inst& I, int type) {
    int t = type < 0 ? -type : type;
    for (int k = I.mat_base; k < I.mat_base + I.n_mat; ++k)
        if (d.mat[k].type == t) return &d.mat[k];
    return nullptr;
}

// ---- smoothing kernels (src/Numeric/kernel.f90) ---------------------------
// Per-target constants: the gradient is dW/dx = g(q) * dx with
// cubic spline (kernel.f90:30-71):
//   q < 1:  g = factor (-2 + 1.5 q) / h^2          = A1 + A2 q
//   q <= 2: g = -factor/2 (2 - q)^2 / h / r         = A3 (2 - q)^2 / r
struct KConst {
    double h, hinv, factor, A1, A2, A3;
    // cubic spline in r (no q): r < h: g = A1 + B1 r;
    // h <= r <= 2h: g = A3 (2 - r/h)^2 / r = C1 / r + C2 r + C3
    double B1, C1, C2, C3;
};
// The FP32 constants of the mixed passes (those of KConst, rounded).
struct KConstF {
    float hinv, factor, A1, A2, A3;
};

// Kernel constants of a system's reference smoothing length (the h of its
// first real particle when it was added).  A target whose h has the same
// bits takes them instead of computing them (five FP64 divisions, which this
// GPU's FP64 pipe runs at about ten times the cost of an FMA): KConst for
// the FP64 passes, KConstF for the mixed ones, and the candidate-test bounds
// of make_target (reach, lo2, hi2) and make_target_m (reach2f).
struct KRef {
    double h;        // +0 when the system has no real particle: matches no target
    int skf;         // kernel the constants belong to
    KConst k;
    KConstF kf;
    double reach;
    float lo2, hi2, reach2f;
};

// Bit-exact conversions on the integer pipes.  On this GPU the conversion
// instructions between float and double issue on the FP64 pipe, at the cost
// of an FP64 FMA; these form the same IEEE 754 results from the bit fields.
// isfinite: the exponent field is not all ones (no FP64 compare).
__device__ __forceinline__ bool finite_d(double x) {
    return ((unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu) != 0x7ffu;
}
// float -> double (exact): the sign, the exponent rebased from 127 to 1023,
// the 23 fraction bits moved up by 29.  Zeros keep their sign; subnormal,
// infinite and NaN inputs take the conversion instruction.
__device__ __forceinline__ double f2d(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    if (e - 1u < 0xfeu)
        return __longlong_as_double((long long)(sgn | ((unsigned long long)(e + 896u) << 52) |
                                                ((unsigned long long)(u & 0x7fffffu) << 29)));
    if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)sgn);
    return (double)f;
}
// double -> float, rounded to nearest even: the top 23 of the 52 fraction
// bits, plus one when the 29 dropped bits are above half, or at half with
// the kept fraction odd (a carry moves into the exponent, as it should).
// Results in the normal float range (exponent 1..253 before rounding, so a
// carry cannot overflow) and zeros take this path; the rest the conversion.
__device__ __forceinline__ float d2f(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;
    if ((unsigned)(e - 1) < 253u) {
        const uint32_t low = (uint32_t)b & 0x1fffffffu;
        uint32_t r = (hi & 0x80000000u) | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
        r += (low > 0x10000000u || (low == 0x10000000u && (r & 1u))) ? 1u : 0u;
        return __uint_as_float(r);
    }
    if ((b << 1) == 0ull) return __uint_as_float(hi & 0x80000000u);
    return __double2float_rn(x);
}

template <int DIM>
__device__ __forceinline__ double cubic_factor(double h) {
    constexpr double PI = 3.141592653589793238462643383279502884;
    if (DIM == 1) return 1.0 / h;
    if (DIM == 2) return 15.0 / ((7.0 * PI) * (h * h));
    return 3.0 / ((2.0 * PI) * ((h * h) * h));
}

template <int DIM>
__device__ __forceinline__ KConst make_kconst(int skf, double h) {
    constexpr double PI = 3.141592653589793238462643383279502884;
    KConst k;
    k.h = h;
    k.hinv = 1.0 / h;
    k.B1 = k.C1 = k.C2 = k.C3 = 0.0;
    if (skf == 1) {
        k.factor = cubic_factor<DIM>(h);
        k.A1 = (k.factor * -2.0) / (h * h);
        k.A2 = (k.factor * 1.5) / (h * h);
        k.A3 = (k.factor * -0.5) / h;
        k.B1 = k.A2 * k.hinv;
        k.C1 = 4.0 * k.A3;
        k.C2 = k.A3 * (k.hinv * k.hinv);
        k.C3 = -4.0 * k.A3 * k.hinv;
    } else if (skf == 2) {
        double b = sqrt(PI) * h, f = b;
        for (int i = 1; i < DIM; ++i) f *= b;
        k.factor = 1.0 / f;
        k.A1 = -2.0 / (h * h);
        k.A2 = k.A3 = 0;
    } else {
        k.factor = DIM == 1 ? 1.0 / (120.0 * h)
                 : DIM == 2 ? 7.0 / ((478.0 * PI) * (h * h))
                            : 1.0 / ((120.0 * PI) * ((h * h) * h));
        k.A1 = k.A2 = k.A3 = 0;
    }
    return k;
}

__device__ __forceinline__ double p4(double a) { double a2 = a * a; return a2 * a2; }
__device__ __forceinline__ double p5(double a) { double a2 = a * a; return (a2 * a2) * a; }

// Cubic-spline gradient factor from r and 1/r (two FMAs per branch, no q).
// Both branches meet at r = h, so the branch choice near q = 1 does not
// change the value beyond rounding.
// a < b (a <= b) for doubles that are +0 or positive: IEEE 754 orders them
// like their bit patterns, so an integer compare decides it exactly and keeps
// the compare off the FP64 pipe, the binding unit of the FP64 pair loops.
__device__ __forceinline__ bool lt_pos(double a, double b) {
    return __double_as_longlong(a) < __double_as_longlong(b);
}
__device__ __forceinline__ bool le_pos(double a, double b) {
    return __double_as_longlong(a) <= __double_as_longlong(b);
}

__device__ __forceinline__ double cubic_g_r(const KConst& k, double r, double rinv) {
    const double gin = fma(k.B1, r, k.A1);
    const double gout = fma(k.C1, rinv, fma(k.C2, r, k.C3));
    return lt_pos(r, k.h) ? gin : gout;   // r >= +0, h > 0
}

// Gradient factor g with dW = g * dx, given q = r/h and 1/r.
__device__ __forceinline__ double kernel_g(int skf, const KConst& k, double q, double rinv) {
    if (skf == 1) {
        double t = 2.0 - q;
        double gin = fma(k.A2, q, k.A1);
        double gout = (k.A3 * (t * t)) * rinv;
        return q < 1.0 ? gin : gout;
    } else if (skf == 2) {
        return q < 3.0 ? (k.factor * exp(-q * q)) * k.A1 : 0.0;
    } else {
        double f = k.factor;
        if (q < 1.0) return (f * ((-120 + 120 * q) - 50 * (q * q))) * (k.hinv * k.hinv);
        if (q < 2.0) return ((f * (-5 * p4(3 - q) + 30 * p4(2 - q))) * k.hinv) * rinv;
        if (q <= 3.0) return ((f * (-5 * p4(3 - q))) * k.hinv) * rinv;
        return 0.0;
    }
}

// Kernel value W(q).
__device__ __forceinline__ double kernel_w(int skf, const KConst& k, double q) {
    if (skf == 1) {
        if (q >= 0 && q < 1) return k.factor * (((2.0 / 3.0) - q * q) + ((q * q) * q) / 2.0);
        if (q >= 1 && q <= 2) { double t = 2 - q; return (k.factor * (1.0 / 6.0)) * ((t * t) * t); }
        return 0.0;
    } else if (skf == 2) {
        return q < 3.0 ? k.factor * exp(-q * q) : 0.0;
    } else {
        double f = k.factor;
        if (q < 1) return f * ((p5(3 - q) - 6 * p5(2 - q)) + 15 * p5(1 - q));
        if (q < 2) return f * (p5(3 - q) - 6 * p5(2 - q));
        if (q <= 3) return f * p5(3 - q);
        return 0.0;
    }
}

// ---- equations of state (src/Physic/eos.f90) ------------------------------
__device__ __forceinline__ double pow_int_or_real(double x, double e) {
    if (e == 7.0) { double x2 = x * x, x4 = x2 * x2; return (x4 * x2) * x; }
    if (e == 4.0) return p4(x);
    if (e == 2.0) return x * x;
    return pow(x, e);
}

// fluid branch of internal_force (internalForce.f90:115-134); updates c for
// the EOS kinds that set the sound speed.
__device__ __forceinline__ void fluid_eos(const DevMaterial* m, double rho, double e, double& p, double& c) {
    if (!m) return;
    switch (m->eos) {
    case SPH_EOS_GAS: {
        double g = m->gamma;
        p = (g - 1) * rho * e;
        c = sqrt(g * p / rho);
    } break;
    case SPH_EOS_TAIT:
        p = m->tait_b * (pow_int_or_real(rho * m->inv_rho0, m->gamma) - 1.0);
        break;
    case SPH_EOS_MORRIS:
        c = (double)0.01f;
        p = (c * c) * rho;
        break;
    case SPH_EOS_LINEAR:
        p = m->k_rho0 * (rho - m->rho0);
        break;
    default: break;
    }
}

// solid branch (internalForce.f90:152-161)
__device__ __forceinline__ void solid_eos(const DevMaterial* m, double rho, double e, double& p) {
    if (!m) return;
    if (m->eos == SPH_EOS_MG_SOLID) {
        double mu = rho * m->inv_rho0 - 1;
        double p1 = m->rho0 * (m->mg_cs * m->mg_cs);
        double p2 = p1 * (1 + 2 * (m->mg_s - 1));
        double p3 = p1 * (2 * (m->mg_s - 1) + 3 * ((m->mg_s - 1) * (m->mg_s - 1)));
        double pH = mu > 0 ? (p1 * mu + p2 * (mu * mu)) + p3 * ((mu * mu) * mu) : p1 * mu;
        p = (1 - (0.5 * m->gamma) * mu) * pH + (m->gamma * rho) * e;
    } else if (m->eos == SPH_EOS_LINEAR) {
        p = m->k_rho0 * (rho - m->rho0);
    }
}

__device__ __forceinline__ bool is_solid_type(int t) { return (t < 0 ? -t : t) > 100; }

// Cell coordinates of a position (clamped into the grid; clamping keeps
// every pair within scale_k*h in adjacent cells).
__device__ __forceinline__ void cell_of(const Grid& g, int dim, const double* x, int* c, bool* clamped) {
    *clamped = false;
    for (int a = 0; a < 3; ++a) {
        if (a >= dim) { c[a] = 0; continue; }
        double t = (x[a] - g.lo[a]) * g.inv_cs;
        int ci;
        if (!(t >= 0.0)) { ci = 0; *clamped = true; }               // also NaN
        else if (t >= (double)g.nc[a]) { ci = g.nc[a] - 1; *clamped = true; }
        else ci = (int)t;
        c[a] = ci;
    }
}

__device__ __forceinline__ int cell_key(const Grid& g, const int* c) {
    return (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
}

// Cell code of the mixed path: the cell coordinates mod 4, one per 4-bit
// field (bits 0-1, 4-5, 8-9).  Accepted neighbours lie in adjacent cells, so
// the mod-4 difference recovers c_i - c_j in {-1, 0, 1} (rel_dx).
__device__ __forceinline__ int cell_code(const int* c) {
    return (c[0] & 3) | ((c[1] & 3) << 4) | ((c[2] & 3) << 8);
}

// FP32 mirrors of one particle for the mixed-precision pair passes.
__device__ __forceinline__ void write_df_mirrors(const Dev& d, const Grid& g, int s, const double4& xm,
                                                 const double4& vr, const double4& eh) {
    const double x[3] = {xm.x, xm.y, xm.z};
    DF r[3];
    for (int a = 0; a < 3; ++a) r[a] = a < d.dim ? df_from(x[a] - g.lo[a]) : DF{0.0f, 0.0f};
    const DF m = df_from(xm.w), v0 = df_from(vr.x), v1 = df_from(vr.y), v2 = df_from(vr.z), rho = df_from(vr.w);
    const DF V = df_from(eh.w), h = df_from(eh.y), c = df_from(eh.z);
    d.pd0[s] = make_float4(r[0].hi, r[1].hi, r[2].hi, m.hi);
    d.pd1[s] = make_float4(r[0].lo, r[1].lo, r[2].lo, m.lo);
    d.vd0[s] = make_float4(v0.hi, v1.hi, v2.hi, rho.hi);
    d.vd1[s] = make_float4(v0.lo, v1.lo, v2.lo, rho.lo);
    d.ed0[s] = make_float4(V.hi, V.lo, h.hi, h.lo);
    float4 e1 = d.ed1[s];
    e1.x = c.hi;
    e1.y = c.lo;
    d.ed1[s] = e1;
}

__device__ __forceinline__ void write_mirrors(const Dev& d, const Grid& g, int s, const double4& xm,
                                              const double4& vr, const double4& eh) {
    if (d.precision == SPH_PREC_DF64) { write_df_mirrors(d, g, s, xm, vr, eh); return; }
    if (d.precision != SPH_PREC_MIXED) return;
    const double x[3] = {xm.x, xm.y, xm.z};
    int c[3];
    bool clamped;
    cell_of(g, d.dim, x, c, &clamped);
    float r[3];
    for (int a = 0; a < 3; ++a)
        r[a] = a < d.dim ? (float)(x[a] - (g.lo[a] + (double)c[a] * g.cs)) : 0.0f;
    d.pr4[s] = make_float4(r[0], r[1], r[2], __int_as_float(cell_code(c)));
    d.vf4[s] = make_float4((float)vr.x, (float)vr.y, (float)vr.z, (float)vr.w);
    d.ef4[s] = make_float4((float)eh.y, (float)eh.z, (float)eh.w, (float)xm.w);
}

// Kahan-compensated FP32 sum.
struct KSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Two Kahan sums advanced together by the packed FP32 instructions (FADD2 /
// FFMA2): per component the operations of KSum, with the compensation kept
// negated (e = -c) so that each step is one packed add or fused multiply-add
// (t - s and y - (t - s) as fma(., -1, .), which rounds like the
// subtraction); add_prod folds the product of a term into the first step.
struct KSum2 {
    float2 s = make_float2(0.0f, 0.0f), e = make_float2(0.0f, 0.0f);
    __device__ __forceinline__ void step(float2 y) {
        const float2 m1 = make_float2(-1.0f, -1.0f);
        const float2 t = __fadd2_rn(s, y);
        const float2 d = __ffma2_rn(s, m1, t);   // t - s
        e = __ffma2_rn(d, m1, y);                // y - (t - s) = -c
        s = t;
    }
    __device__ __forceinline__ void add(float2 x) { step(__fadd2_rn(x, e)); }                   // y = x - c
    __device__ __forceinline__ void add_prod(float2 p, float2 q) { step(__ffma2_rn(p, q, e)); }  // y = p q - c
    __device__ __forceinline__ double x() const { return (double)s.x + (double)e.x; }
    __device__ __forceinline__ double y() const { return (double)s.y + (double)e.y; }
    // the same sums rounded to FP32: s + e rounds like (float)x(), since the
    // compensation is below an ulp of s (the double sum is exact, or e is too
    // small to move the rounding)
    __device__ __forceinline__ float xf() const { return s.x + e.x; }
    __device__ __forceinline__ float yf() const { return s.y + e.y; }
};

// ---- kernel gradient correction (kernelGradientCorrection.f90:8-51) -------
// The reference solves A_i x = dW_ij for every neighbour with its pivoted
// elimination MCPE (tools.f90:287-354): the pivot row of each column is
// chosen first, on the matrix as it stands after the earlier swaps; the rows
// are then eliminated without further pivoting, and a row that becomes
// exactly zero ends the solve with the gradient unchanged.  A_i is the same
// for all neighbours of i, so its swaps, multipliers and upper triangle are
// computed once per target and applied per pair with the same operations in
// the same order (no FMA contraction).
template <int DIM>
struct KgcLayout {
    static constexpr int PERM = 0;                             // DIM pivot rows
    static constexpr int FLAG = DIM;                           // 1: a row vanished
    static constexpr int MULT = DIM + 1;                       // DIM (DIM - 1) / 2 multipliers
    static constexpr int UPPER = MULT + DIM * (DIM - 1) / 2;   // row-major upper triangle
    static constexpr int SIZE = UPPER + DIM * (DIM + 1) / 2;
    static constexpr __host__ __device__ int upper(int i, int j) {  // j >= i
        return UPPER + i * DIM - (i * (i - 1)) / 2 + (j - i);
    }
};
constexpr int KGC_STRIDE = 16;
static_assert(KgcLayout<3>::SIZE <= KGC_STRIDE, "kernel-correction factors");

template <int DIM>
__device__ __forceinline__ void kgc_factor(double A[DIM][DIM], double* out) {
    using L = KgcLayout<DIM>;
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
        int p = i;
#pragma unroll
        for (int j = i + 1; j < DIM; ++j)
            if (fabs(A[p][i]) < fabs(A[j][i])) p = j;
#pragma unroll
        for (int q = i + 1; q < DIM; ++q)
            if (p == q) {
#pragma unroll
                for (int c = 0; c < DIM; ++c) { const double t = A[i][c]; A[i][c] = A[q][c]; A[q][c] = t; }
            }
        out[L::PERM + i] = (double)p;
    }
    out[L::FLAG] = 0.0;
    int m = 0;
#pragma unroll
    for (int i = 0; i < DIM - 1; ++i)
#pragma unroll
        for (int j = i + 1; j < DIM; ++j) {
            const double buffer = __ddiv_rn(A[j][i], A[i][i]);
            double temp = 0.0;
#pragma unroll
            for (int k = i; k < DIM; ++k) {
                A[j][k] = __dsub_rn(A[j][k], __dmul_rn(A[i][k], buffer));
                temp = __dadd_rn(temp, __dmul_rn(A[j][k], A[j][k]));
            }
            out[L::MULT + m++] = buffer;
            if (temp == 0.0) out[L::FLAG] = 1.0;
        }
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int k = i; k < DIM; ++k) out[L::upper(i, k)] = A[i][k];
}

// g <- A_i^-1 g with the stored factors (the gradient stays if A_i was
// found singular).
template <int DIM>
__device__ __forceinline__ void kgc_apply(const double* f, double* g) {
    using L = KgcLayout<DIM>;
    if (f[L::FLAG] != 0.0) return;
    double B[DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a) B[a] = g[a];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
        const int p = (int)f[L::PERM + i];
#pragma unroll
        for (int q = i + 1; q < DIM; ++q)
            if (p == q) { const double t = B[i]; B[i] = B[q]; B[q] = t; }
    }
    int m = 0;
#pragma unroll
    for (int i = 0; i < DIM - 1; ++i)
#pragma unroll
        for (int j = i + 1; j < DIM; ++j) B[j] = __dsub_rn(B[j], __dmul_rn(B[i], f[L::MULT + m++]));
    double X[DIM];
    X[DIM - 1] = __ddiv_rn(B[DIM - 1], f[L::upper(DIM - 1, DIM - 1)]);
#pragma unroll
    for (int i = DIM - 2; i >= 0; --i) {
#pragma unroll
        for (int j = DIM - 1; j >= i + 1; --j) B[i] = __dsub_rn(B[i], __dmul_rn(f[L::upper(i, j)], X[j]));
        X[i] = __ddiv_rn(B[i], f[L::upper(i, i)]);
    }
#pragma unroll
    for (int a = 0; a < DIM; ++a) g[a] = X[a];
}

// ---- FP64 reciprocal for the pair physics ----------------------------------
// An FP32 hardware estimate refined by one Newton-Raphson step in FP64,
// y1 = y0 + y0 (1 - x y0): the relative error after the step is about e0^2
// for an estimate error e0 (below 1e-7), i.e. about 1e-14, far below the
// 1e-10 parity bar, at two FP64 operations instead of a full division.
// Outside the FP32 normal range the FP64 division is used.
__device__ __forceinline__ double rcp_nr(double x) {
    const float xf = (float)x;
    const float ax = fabsf(xf);
    if (!(ax > 1e-30f && ax < 1e30f)) return 1.0 / x;
    const double y = (double)(1.0f / xf);
    const double e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// ---- warp helpers ----------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(SPH_FULL_MASK, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(SPH_FULL_MASK, v, o));
    return v;
}
__device__ __forceinline__ int warp_max_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(SPH_FULL_MASK, v, o));
    return v;
}
__device__ __forceinline__ int warp_min_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(SPH_FULL_MASK, v, o));
    return v;
}

}  // namespace sph
