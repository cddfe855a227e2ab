// sph_oracle.cpp — CPU restatement of mySPH's per-step particle path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GPU
// library and, built with OpenMP, the timed CPU baseline.  Nothing in the
// product (mysph_gb300/, libsphgpu.so) links, loads or calls it; only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
//
// PARITY UNPINNED: the reference (Fortran 2018 + OpenMP) cannot be compiled
// in this environment (no Fortran compiler, and its toml-f dependency is not
// vendored) and ships no golden vectors or known-answer tests for this path.
// This restatement is therefore checked against analytic known answers and
// a brute-force O(N^2) neighbour enumeration (tests/), not against outputs
// of the reference itself.
//
// Every routine follows the cited reference routine in operation order,
// including its quirks, so that FP64 results agree to rounding:
//   - single precision literals of the reference (e.g. `1.2`, `9.81`, `0.01`
//     without _8) are double-rounded-from-float here as well;
//   - `x**0.5` / `x**p` with real exponents are std::pow calls, integer
//     powers are products, as gfortran emits them;
//   - the reference's OpenMP data races (shared J2/SigmaY/cntemp, `save`
//     variables eta/chi/factor_c) are resolved to serial semantics.
// Built twice from the same source: serial (-O2 -ffp-contract=off, the
// oracle) and -fopenmp (-O3 -ffp-contract=off, the CPU baseline).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/sph_gpu.h"

namespace {

constexpr double PI = 3.141592653589793238462643383279502884;  // acos(-1._8), src/tools.f90:8
inline double f32(double v) { return (double)(float)v; }  // a default-real literal

struct Orc {
    sph_params prm{};
    int dim = 2;
    int64_t n_real = 0, n_wall = 0, N = 0;
    // particle data (src/Initialize/SPH.f90:6-25), SoA, Fortran layouts
    std::vector<double> x, v, disp;              // N*dim
    std::vector<double> mass, rho, p, e, c, h;   // N
    std::vector<double> visc, divx, divv;        // N
    std::vector<int32_t> type, state, boundary;  // N
    std::vector<double> stress;                  // N*dim*dim
    // neighbour lists stored per target (neighborList, w, dwdx)
    std::vector<std::vector<int32_t>> nl;
    std::vector<std::vector<double>> w, dwdx;
    // leap-frog arrays (src/TimeIntegration/timeIntegration.f90:38-66)
    std::vector<double> prev_v, prev_rho, prev_e;
    std::vector<double> dvdt, drhodt, dedt;      // Delta
    std::vector<double> shear, shear_prev, dsdt; // N*dim*dim
    std::vector<double> aver_v;                  // N*dim
    // per-module outputs of the last single_step (parity exports)
    std::vector<double> indvdt, indedt, exdvdt, avdvdt, avdedt, asdvdt, ahdedt;
    std::vector<double> edot, rdot, tdsdt;
    int64_t step = 0;
    double time = 0, max_courant = 0, aver_courant = 0;
    // 0: the reference's band of int(h/cell)+1 cells; 1: a band that covers
    // scale_k*h (exact r < scale_k*h sets on every grid; test option)
    int search_mode = 0;
};

inline const sph_material* material_of(const Orc& o, int32_t type) {
    int32_t t = type < 0 ? -type : type;
    for (int k = 0; k < o.prm.n_materials && k < SPH_MAX_MATERIALS; ++k)
        if (o.prm.materials[k].type == t) return &o.prm.materials[k];
    return nullptr;
}

inline int scale_k_of(int skf) {  // asymmetricSearch.f90:178-185
    if (skf == 1) return 2;
    if (skf == 2 || skf == 3) return 3;
    return 1;
}

// ---- kernels: src/Numeric/kernel.f90 ------------------------------------
// cubic_spline_function, kernel.f90:30-71
void cubic(int dim, double r, const double* dx, double hsml, double& w, double* dw) {
    double q = r / hsml;
    double factor = 0;
    w = 0;
    for (int d = 0; d < dim; ++d) dw[d] = 0;
    if (dim == 1) factor = 1.0 / hsml;
    else if (dim == 2) factor = 15.0 / ((7.0 * PI) * (hsml * hsml));
    else if (dim == 3) factor = 3.0 / ((2.0 * PI) * ((hsml * hsml) * hsml));
    if (q >= 0 && q < 1) {
        w = factor * (((2.0 / 3.0) - q * q) + ((q * q) * q) / 2.0);
        double g = (factor * (-2.0 + 1.5 * q)) / (hsml * hsml);
        for (int d = 0; d < dim; ++d) dw[d] = g * dx[d];
    } else if (q >= 1 && q <= 2) {
        double t = 2 - q;
        w = (factor * (1.0 / 6.0)) * ((t * t) * t);
        double g = ((factor * (-1.0 / 2.0)) * (t * t)) / hsml;
        for (int d = 0; d < dim; ++d) dw[d] = g * (dx[d] / r);
    }
}

// gauss_kernel_function, kernel.f90:73-107
void gauss(int dim, double r, const double* dx, double hsml, double& w, double* dw) {
    double q = r / hsml;
    double b = std::sqrt(PI) * hsml, f = b;
    for (int k = 1; k < dim; ++k) f *= b;
    double factor = 1.0 / f;
    w = 0;
    for (int d = 0; d < dim; ++d) dw[d] = 0;
    if (q >= 0 && q < 3) {
        w = factor * std::exp(-q * q);
        for (int d = 0; d < dim; ++d) dw[d] = w * ((-2.0 * dx[d]) / (hsml * hsml));
    }
}

inline double p5(double a) { double a2 = a * a; return (a2 * a2) * a; }
inline double p4(double a) { double a2 = a * a; return a2 * a2; }

// quintic_kernel_function, kernel.f90:109-154
void quintic(int dim, double r, const double* dx, double hsml, double& w, double* dw) {
    double q = r / hsml;
    double factor = 0;
    w = 0;
    for (int d = 0; d < dim; ++d) dw[d] = 0;
    if (dim == 1) factor = 1.0 / (120.0 * hsml);
    else if (dim == 2) factor = 7.0 / ((478.0 * PI) * (hsml * hsml));
    else if (dim == 3) factor = 1.0 / ((120.0 * PI) * ((hsml * hsml) * hsml));
    if (q >= 0 && q < 1) {
        w = factor * ((p5(3 - q) - 6 * p5(2 - q)) + 15 * p5(1 - q));
        double g = (factor * ((-120 + 120 * q) - 50 * (q * q))) / (hsml * hsml);
        for (int d = 0; d < dim; ++d) dw[d] = g * dx[d];
    } else if (q >= 1 && q < 2) {
        w = factor * (p5(3 - q) - 6 * p5(2 - q));
        double g = (factor * (-5 * p4(3 - q) + 30 * p4(2 - q))) / hsml;
        for (int d = 0; d < dim; ++d) dw[d] = g * (dx[d] / r);
    } else if (q >= 2 && q <= 3) {
        w = factor * p5(3 - q);
        double g = (factor * (-5 * p4(3 - q))) / hsml;
        for (int d = 0; d < dim; ++d) dw[d] = g * (dx[d] / r);
    }
}

// kernel dispatch, kernel.f90:8-28
inline void kernel(int skf, int dim, double r, const double* dx, double hsml, double& w, double* dw) {
    if (skf == 1) cubic(dim, r, dx, hsml, w, dw);
    else if (skf == 2) gauss(dim, r, dx, hsml, w, dw);
    else if (skf == 3) quintic(dim, r, dx, hsml, w, dw);
}

// ---- equations of state: src/Physic/eos.f90 ------------------------------
// Fluid branch (abs(Type) <= 100) of internal_force, internalForce.f90:115-134.
void fluid_eos(const sph_material* m, double rho, double e, double& p, double& c) {
    if (!m) return;
    switch (m->eos) {
    case SPH_EOS_GAS: {  // gas_eos, eos.f90:9-18 (gamma = 1.4 single literal)
        double g = m->gamma;
        p = (g - 1) * rho * e;
        c = std::sqrt(g * p / rho);
    } break;
    case SPH_EOS_TAIT: {  // arti_water_eos_1, eos.f90:23-53
        double b = ((m->c0 * m->c0) * m->rho0) / m->gamma;
        p = b * (std::pow(rho / m->rho0, m->gamma) - 1);
    } break;
    case SPH_EOS_MORRIS: {  // arti_water_eos_2, eos.f90:57-64
        c = f32(0.01);
        p = (c * c) * rho;
    } break;
    case SPH_EOS_LINEAR: {  // same form as the oil EOS, eos.f90:149-157
        p = (m->K / m->rho0) * (rho - m->rho0);
    } break;
    default: break;
    }
}

// Solid branch, internalForce.f90:152-161.
void solid_eos(const sph_material* m, double rho, double e, double& p) {
    if (!m) return;
    if (m->eos == SPH_EOS_MG_SOLID) {  // mie_gruneisen_eos_of_armcoIron, eos.f90:180-215
        double mu = rho / m->rho0 - 1;
        double p1 = m->rho0 * (m->mg_cs * m->mg_cs);
        double p2 = p1 * (1 + 2 * (m->mg_s - 1));
        double p3 = p1 * (2 * (m->mg_s - 1) + 3 * ((m->mg_s - 1) * (m->mg_s - 1)));
        double pH = mu > 0 ? (p1 * mu + p2 * (mu * mu)) + p3 * ((mu * mu) * mu) : p1 * mu;
        p = (1 - (0.5 * m->gamma) * mu) * pH + (m->gamma * rho) * e;
    } else if (m->eos == SPH_EOS_LINEAR) {  // arti_eos_of_102/103/Aluminium, eos.f90:219-248
        double cc = m->K / m->rho0;
        p = cc * (rho - m->rho0);
    }
}

// ---- NNPS: BGGS, src/NNPS/asymmetricSearch.f90 ---------------------------
struct Grid {
    int cellNum[3] = {1, 1, 1};
    double maxC[3] = {0, 0, 0}, minC[3] = {0, 0, 0};
    std::vector<std::vector<int32_t>> cells;  // x fastest
    bool locate(const Orc& o, int64_t i, int* cell) const {  // locate, :27-47
        for (int d = 0; d < o.dim; ++d) {
            double xd = o.x[i * o.dim + d];
            if (!(xd <= maxC[d]) || !(xd >= minC[d])) return false;  // "particle out of range"
            cell[d] = (int)(((xd - minC[d]) / (maxC[d] - minC[d])) * cellNum[d] + 1);
        }
        for (int d = o.dim; d < 3; ++d) cell[d] = 1;
        return true;
    }
    std::vector<int32_t>& at(int cx, int cy, int cz) {
        return cells[((size_t)(cz - 1) * cellNum[1] + (cy - 1)) * cellNum[0] + (cx - 1)];
    }
    const std::vector<int32_t>& at(int cx, int cy, int cz) const {
        return cells[((size_t)(cz - 1) * cellNum[1] + (cy - 1)) * cellNum[0] + (cx - 1)];
    }
};

// grid_t%initialize, asymmetricSearch.f90:49-158 (serial in the reference)
int grid_init(const Orc& o, Grid& g) {
    const double GMR = f32(1.2);  // real(8), parameter :: GMR = 1.2
    const int NPG = 3;
    const int dim = o.dim;
    const int64_t ntotal = o.N;
    double mx[3], mn[3];
    for (int d = 0; d < 3; ++d) { mx[d] = -std::numeric_limits<double>::max(); mn[d] = std::numeric_limits<double>::max(); }
    for (int64_t i = 0; i < ntotal; ++i)
        for (int d = 0; d < dim; ++d) {
            double xd = o.x[i * dim + d];
            if (xd > mx[d]) mx[d] = xd;
            if (xd < mn[d]) mn[d] = xd;
        }
    double delta[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) delta[d] = mx[d] - mn[d];
    for (int d = 0; d < dim; ++d) {
        g.maxC[d] = mx[d] + (GMR - 1) * delta[d];
        g.minC[d] = mn[d] - (GMR - 1) * delta[d];
    }
    if (dim == 1) {
        g.cellNum[0] = (int)std::min<int64_t>(ntotal / NPG + 1, 1000);
    } else if (dim == 2) {
        g.cellNum[0] = std::min((int)std::pow(((double)ntotal * delta[0]) / (delta[1] * NPG), 1.0 / 2) + 1, 1000);
        g.cellNum[1] = std::min((int)(g.cellNum[0] * delta[1] / delta[0]) + 1, 1000);
    } else {
        g.cellNum[0] = std::min((int)std::pow((((double)ntotal * delta[0]) * delta[0]) / ((delta[1] * delta[2]) * NPG), 1.0 / 3) + 1, 1000);
        g.cellNum[1] = std::min((int)(g.cellNum[0] * delta[1] / delta[0]) + 1, 1000);
        g.cellNum[2] = std::min((int)(g.cellNum[0] * delta[2] / delta[0]) + 1, 1000);
    }
    for (int d = dim; d < 3; ++d) g.cellNum[d] = 1;
    g.cells.assign((size_t)g.cellNum[0] * g.cellNum[1] * g.cellNum[2], {});
    for (int64_t i = 0; i < ntotal; ++i) {
        if (o.state[i] == -1) continue;
        int cell[3];
        if (!g.locate(o, i, cell)) return SPH_E_RANGE;
        g.at(cell[0], cell[1], cell[2]).push_back((int32_t)i);
    }
    return SPH_OK;
}

// BGGS, asymmetricSearch.f90:160-257, Targets = P(1:ntotal), Sources = P(1:N),
// skipItsSelf = .true. (singleStep.f90:84).
int bggs(Orc& o) {
    Grid g;
    int st = grid_init(o, g);
    if (st) return st;
    const int dim = o.dim, skf = o.prm.skf;
    const int scale_k = scale_k_of(skf);
    const int64_t nt = o.n_real;
    o.nl.resize(nt); o.w.resize(nt); o.dwdx.resize(nt);
    int err = 0;
#ifdef _OPENMP
    int nth = omp_get_max_threads();
    int chunk = (int)std::max<int64_t>(1, nt / nth);
#pragma omp parallel for schedule(dynamic, chunk) reduction(| : err)
#endif
    for (int64_t i = 0; i < nt; ++i) {
        o.nl[i].clear(); o.w[i].clear(); o.dwdx[i].clear();
        if (o.state[i] == -1) continue;
        int cell[3];
        if (!g.locate(o, i, cell)) { err = 1; continue; }
        int maxCell[3] = {1, 1, 1}, minCell[3] = {1, 1, 1};
        double hi = o.h[i];
        for (int d = 0; d < dim; ++d) {
            int per = (int)(hi / (g.maxC[d] - g.minC[d]) * g.cellNum[d]) + 1;
            if (o.search_mode == 1)
                per = (int)std::ceil(hi * scale_k / (g.maxC[d] - g.minC[d]) * g.cellNum[d]) + 1;
            maxCell[d] = std::min(cell[d] + per, g.cellNum[d]);
            minCell[d] = std::max(cell[d] - per, 1);
        }
        double dx[3], w, dw[3];
        for (int zc = minCell[2]; zc <= maxCell[2]; ++zc)
            for (int yc = minCell[1]; yc <= maxCell[1]; ++yc)
                for (int xc = minCell[0]; xc <= maxCell[0]; ++xc) {
                    const auto& lst = g.at(xc, yc, zc);
                    for (int32_t j : lst) {
                        if (o.state[j] == -1) continue;
                        if (i == j) continue;
                        dx[0] = o.x[i * dim] - o.x[(int64_t)j * dim];
                        double dr = dx[0] * dx[0];
                        for (int d = 1; d < dim; ++d) {
                            dx[d] = o.x[i * dim + d] - o.x[(int64_t)j * dim + d];
                            dr = dr + dx[d] * dx[d];
                        }
                        double r = std::pow(dr, 0.5);
                        double mhsml = hi;
                        if (r < mhsml * scale_k) {
                            o.nl[i].push_back(j + 0);
                            kernel(skf, dim, r, dx, mhsml, w, dw);
                            o.w[i].push_back(w);
                            for (int d = 0; d < dim; ++d) o.dwdx[i].push_back(dw[d]);
                        }
                    }
                }
    }
    return err ? SPH_E_RANGE : SPH_OK;
}

// ---- density: src/Physic/density.f90 -------------------------------------
// con_density, density.f90:83-107
void con_density(Orc& o) {
    const int dim = o.dim;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < o.n_real; ++i) {
        double acc = 0;
        const auto& L = o.nl[i];
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            double s = 0;
            for (int d = 0; d < dim; ++d) s = s + (o.v[i * dim + d] - o.v[j * dim + d]) * o.dwdx[i][k * dim + d];
            acc = acc + ((o.mass[j] * s) * o.rho[i]) / o.rho[j];
        }
        o.drhodt[i] = acc;
    }
}

// con_density_riemann, density.f90:110-148 (SPH = 3): the PVRS velocity of
// each pair, with the neighbour's sound speed on both sides (Z_l = rho_i c_j)
// and the pressures of the previous EOS
void con_density_riemann(Orc& o) {
    const int dim = o.dim;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < o.n_real; ++i) {
        double acc = 0;
        const auto& L = o.nl[i];
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            double Zl = o.rho[i] * o.c[j];
            double Zr = o.rho[j] * o.c[j];
            double e[3], nrm = 0;
            for (int d = 0; d < dim; ++d) { e[d] = o.x[j * dim + d] - o.x[i * dim + d]; nrm = nrm + e[d] * e[d]; }
            nrm = std::sqrt(nrm);
            for (int d = 0; d < dim; ++d) e[d] = e[d] / nrm;
            double vl = 0, vr = 0;
            for (int d = 0; d < dim; ++d) vl = vl + o.v[i * dim + d] * e[d];
            for (int d = 0; d < dim; ++d) vr = vr + o.v[j * dim + d] * e[d];
            double vij = (Zl * vl + Zr * vr + (o.p[i] - o.p[j])) / (Zl + Zr);
            double dot = 0;
            for (int d = 0; d < dim; ++d) {
                double vs = vij * e[d] + ((o.v[i * dim + d] + o.v[j * dim + d]) / 2 - ((vl + vr) / 2) * e[d]);
                dot = dot + (o.v[i * dim + d] - vs) * o.dwdx[i][k * dim + d];
            }
            acc = acc + 2 * o.rho[i] * o.mass[j] / o.rho[j] * dot;
        }
        o.drhodt[i] = acc;
    }
}

// sum_density, density.f90:10-80 (N = ntotal)
void sum_density(Orc& o) {
    const int dim = o.dim;
    const int64_t n = o.n_real;
    const bool norm = o.prm.flags & SPH_F_NORM_DENSITY;
    std::vector<double> wi(n, 0.0);
    double zero[3] = {0, 0, 0}, hv[3];
    if (norm) {
        for (int64_t i = 0; i < n; ++i)
            if (o.divx[i] < 1.5) {
                double self;
                kernel(o.prm.skf, dim, 0.0, zero, o.h[i], self, hv);
                wi[i] = o.mass[i] / o.rho[i] * self;
            }
        for (int64_t i = 0; i < n; ++i)
            if (o.divx[i] < 1.5)
                for (size_t k = 0; k < o.nl[i].size(); ++k) {
                    int64_t j = o.nl[i][k];
                    wi[i] = wi[i] + o.mass[j] / o.rho[j] * o.w[i][k];
                }
    }
    std::vector<double> newrho(n);
    for (int64_t i = 0; i < n; ++i) {
        double self;
        kernel(o.prm.skf, dim, 0.0, zero, o.h[i], self, hv);
        newrho[i] = o.mass[i] * self;
    }
    // The reference updates P(i)%Density in place while later targets read
    // P(j)%Mass only, so the order of updates does not matter.
    for (int64_t i = 0; i < n; ++i)
        for (size_t k = 0; k < o.nl[i].size(); ++k) {
            int64_t j = o.nl[i][k];
            newrho[i] = newrho[i] + o.mass[j] * o.w[i][k];
        }
    for (int64_t i = 0; i < n; ++i) {
        o.rho[i] = newrho[i];
        if (norm && o.divx[i] < 1.5) o.rho[i] = o.rho[i] / wi[i];
    }
}

// ---- kernel gradient correction: kernelGradientCorrection.f90:8-51 -------
// MCPE (tools.f90:287-354): the pivot of every column is chosen first, on
// the matrix as it stands after the earlier swaps, then the rows are
// eliminated without further pivoting; a row that becomes exactly zero
// returns early and leaves X (the gradient) as it was.
void mcpe(int n, double* A, double* B, double* X) {  // A row-major n x n
    for (int i = 0; i < n; ++i) {
        int p = i;
        for (int j = i + 1; j < n; ++j)
            if (std::abs(A[p * n + i]) < std::abs(A[j * n + i])) p = j;
        for (int j = 0; j < n; ++j) std::swap(A[i * n + j], A[p * n + j]);
        std::swap(B[i], B[p]);
    }
    for (int i = 0; i < n - 1; ++i)
        for (int j = i + 1; j < n; ++j) {
            const double buffer = A[j * n + i] / A[i * n + i];
            double temp = 0;
            for (int k = i; k < n; ++k) {
                A[j * n + k] = A[j * n + k] - A[i * n + k] * buffer;
                temp = temp + A[j * n + k] * A[j * n + k];
            }
            B[j] = B[j] - B[i] * buffer;
            if (temp == 0) return;
        }
    X[n - 1] = B[n - 1] / A[(n - 1) * n + n - 1];
    for (int i = n - 2; i >= 0; --i) {
        for (int j = n - 1; j >= i + 1; --j) B[i] = B[i] - A[i * n + j] * X[j];
        X[i] = B[i] / A[i * n + i];
    }
}

void kernel_correction(Orc& o) {
    const int dim = o.dim;
    const int64_t nt = o.n_real;
    std::vector<double> A(nt * dim * dim, 0.0);  // A(d, e, i) at [i][d][e]
    for (int64_t i = 0; i < nt; ++i) {
        if (o.type[i] <= 100) continue;
        for (size_t k = 0; k < o.nl[i].size(); ++k) {
            const int64_t j = o.nl[i][k];
            if ((std::abs(o.type[i]) - 100) * (std::abs(o.type[j]) - 100) < 0) continue;
            for (int d = 0; d < dim; ++d)
                for (int e = 0; e < dim; ++e)
                    A[(i * dim + d) * dim + e] = A[(i * dim + d) * dim + e] +
                        (o.x[j * dim + e] - o.x[i * dim + e]) * o.dwdx[i][k * dim + d] * o.mass[j] / o.rho[j];
        }
    }
    double T[9], B[3];
    for (int64_t i = 0; i < nt; ++i)
        for (size_t k = 0; k < o.nl[i].size(); ++k) {
            std::copy(&A[i * dim * dim], &A[i * dim * dim] + dim * dim, T);
            std::copy(&o.dwdx[i][k * dim], &o.dwdx[i][k * dim] + dim, B);
            mcpe(dim, T, B, &o.dwdx[i][k * dim]);
        }
}

// ---- divergence: src/Numeric/divergence.f90:6-29 -------------------------
void divergence(Orc& o) {
    const int dim = o.dim;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < o.n_real; ++i) {
        double ax = 0, av = 0;
        const auto& L = o.nl[i];
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            double sx = 0, sv = 0;
            for (int d = 0; d < dim; ++d) {
                sx = sx + (o.x[j * dim + d] - o.x[i * dim + d]) * o.dwdx[i][k * dim + d];
                sv = sv + (o.v[j * dim + d] - o.v[i * dim + d]) * o.dwdx[i][k * dim + d];
            }
            ax = ax + o.mass[j] / o.rho[j] * sx;
            av = av + o.mass[j] / o.rho[j] * sv;
        }
        o.divx[i] = ax;
        o.divv[i] = av;
    }
}

// With SPH_F_FSI_FLUID_VISCOUS, a solid neighbour contributes no viscous term
// to a fluid particle.  Without it (the reference), the fluid adds
// P(j)%Viscosity*edot(:,:,j) of a solid j (internalForce.f90:242-243), whose
// Viscosity is the shear modulus (viscosity.f90:21-28).
inline bool solid_j_dropped(const Orc& o, int64_t j) {
    return (o.prm.flags & SPH_F_FSI_FLUID_VISCOUS) && std::abs(o.type[j]) > 100;
}

// ---- internal force: src/Physic/internalForce.f90:10-342 -----------------
void internal_force(Orc& o) {
    const int dim = o.dim, D2 = dim * dim;
    const int64_t N = o.N, nt = o.n_real;
    const bool viscw = o.prm.flags & SPH_F_VISCOSITY;
    o.edot.assign(N * D2, 0.0);
    o.rdot.assign(N * D2, 0.0);
    o.tdsdt.assign(N, 0.0);
    auto E = [&](int64_t i, int d, int dd) -> double& { return o.edot[i * D2 + dd * dim + d]; };
    auto R = [&](int64_t i, int d, int dd) -> double& { return o.rdot[i * D2 + dd * dim + d]; };
    auto S = [&](std::vector<double>& a, int64_t i, int d, int dd) -> double& { return a[i * D2 + dd * dim + d]; };

    // viscosity table, src/Physic/viscosity.f90:5-35 (internalForce.f90:45)
    if (viscw)
        for (int64_t i = 0; i < N; ++i) {
            const sph_material* m = material_of(o, o.type[i]);
            o.visc[i] = m ? m->eta : 0.0;
        }

    // strain-rate loops over all particles, internalForce.f90:48-100
    if (viscw) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < nt; ++i) {  // walls (i > ntotal) have no neighbours
            const auto& L = o.nl[i];
            const double* DW = o.dwdx[i].data();
            double dv[3];
            if (std::abs(o.type[i]) <= 100) {  // fluid, :56-77
                for (size_t k = 0; k < L.size(); ++k) {
                    int64_t j = L[k];
                    for (int d = 0; d < dim; ++d) dv[d] = o.v[j * dim + d] - o.v[i * dim + d];
                    for (int d = 0; d < dim; ++d)
                        for (int dd = 0; dd < dim; ++dd) {
                            E(i, d, dd) = E(i, d, dd) + o.mass[j] / o.rho[j] * dv[d] * DW[k * dim + dd];
                            E(i, dd, d) = E(i, dd, d) + o.mass[j] / o.rho[j] * dv[dd] * DW[k * dim + d];
                            if (d == dd)
                                for (int ddd = 0; ddd < dim; ++ddd)
                                    E(i, d, d) = E(i, d, d) - 2.0 / 3 * o.mass[j] / o.rho[j] * dv[ddd] * DW[k * dim + ddd];
                        }
                }
            } else {  // solid, :82-95
                for (size_t k = 0; k < L.size(); ++k) {
                    int64_t j = L[k];
                    for (int d = 0; d < dim; ++d) dv[d] = o.v[j * dim + d] - o.v[i * dim + d];
                    for (int d = 0; d < dim; ++d)
                        for (int dd = 0; dd < dim; ++dd) {
                            double vab = 0.5 * o.mass[j] / o.rho[j] * dv[d] * DW[k * dim + dd];
                            double vba = 0.5 * o.mass[j] / o.rho[j] * dv[dd] * DW[k * dim + d];
                            E(i, d, dd) = E(i, d, dd) + (vab + vba);
                            R(i, d, dd) = R(i, d, dd) + (vab - vba);
                        }
                }
            }
        }
    }

    // EOS, viscous entropy, deviatoric stress rate, stress: :103-189 (all N)
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < N; ++i) {
        const sph_material* m = material_of(o, o.type[i]);
        if (std::abs(o.type[i]) <= 100) {
            if (viscw) {
                double s = 0;
                for (int dd = 0; dd < dim; ++dd)
                    for (int d = 0; d < dim; ++d) s = s + E(i, d, dd) * E(i, d, dd);
                o.tdsdt[i] = 0.5 * o.visc[i] / o.rho[i] * s;
            }
            fluid_eos(m, o.rho[i], o.e[i], o.p[i], o.c[i]);
        } else {
            double aux = 0;
            for (int d = 0; d < dim; ++d) aux = aux + E(i, d, d);
            aux = aux / 3;
            double ae[9];
            for (int dd = 0; dd < dim; ++dd)
                for (int d = 0; d < dim; ++d) ae[dd * dim + d] = E(i, d, dd);
            for (int d = 0; d < dim; ++d) ae[d * dim + d] = ae[d * dim + d] - aux;
            double s = 0;
            for (int dd = 0; dd < dim; ++dd)
                for (int d = 0; d < dim; ++d) s = s + S(o.shear, i, d, dd) * ae[dd * dim + d];
            o.tdsdt[i] = s / o.rho[i];
            solid_eos(m, o.rho[i], o.e[i], o.p[i]);
            for (int d = 0; d < dim; ++d)
                for (int dd = 0; dd < dim; ++dd) {
                    double t = 2 * o.visc[i] * ae[dd * dim + d];
                    for (int ddd = 0; ddd < dim; ++ddd)
                        t = t + S(o.shear, i, d, ddd) * R(i, dd, ddd) + S(o.shear, i, dd, ddd) * R(i, d, ddd);
                    S(o.dsdt, i, d, dd) = t;
                }
            for (int d = 0; d < dim; ++d) {
                for (int dd = 0; dd < dim; ++dd) S(o.stress, i, d, dd) = S(o.shear, i, d, dd);
                S(o.stress, i, d, d) = S(o.stress, i, d, d) - o.p[i];
            }
        }
    }

    // momentum / energy pair loops, :194-329
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < nt; ++i) {
        double* dvdt = &o.indvdt[i * dim];
        double dedt = 0;
        for (int d = 0; d < dim; ++d) dvdt[d] = 0;
        const auto& L = o.nl[i];
        const double* DW = o.dwdx[i].data();
        if (o.prm.pa_sph == 1) {
            if (std::abs(o.type[i]) <= 100) {  // :199-221
                for (size_t k = 0; k < L.size(); ++k) {
                    int64_t j = L[k];
                    double rhoij = 1.0 / (o.rho[i] * o.rho[j]);
                    double aux = (o.p[i] + o.p[j]) * rhoij;
                    for (int d = 0; d < dim; ++d) {
                        double mm = 0;
                        for (int dd = 0; dd < dim; ++dd)
                            mm = mm + (o.visc[i] * E(i, d, dd) + o.visc[j] * E(j, d, dd)) * DW[k * dim + dd];
                        dvdt[d] = dvdt[d] + o.mass[j] * (-aux * DW[k * dim + d] + mm * rhoij);
                    }
                    double dot = 0;
                    for (int d = 0; d < dim; ++d) dot = dot + (o.v[i * dim + d] - o.v[j * dim + d]) * DW[k * dim + d];
                    dedt = dedt + o.mass[j] * aux * dot;
                }
            }
        } else if (o.prm.pa_sph == 3) {
            if (std::abs(o.type[i]) <= 100) {  // :277-322
                for (size_t k = 0; k < L.size(); ++k) {
                    int64_t j = L[k];
                    double rhoij = 1.0 / (o.rho[i] * o.rho[j]);
                    double Zl = o.rho[i] * o.c[i];
                    double Zr = o.rho[j] * o.c[j];
                    double e[3], nrm = 0;
                    for (int d = 0; d < dim; ++d) { e[d] = o.x[j * dim + d] - o.x[i * dim + d]; nrm = nrm + e[d] * e[d]; }
                    nrm = std::sqrt(nrm);
                    for (int d = 0; d < dim; ++d) e[d] = e[d] / nrm;
                    double vl = 0, vr = 0;
                    for (int d = 0; d < dim; ++d) vl = vl + o.v[i * dim + d] * e[d];
                    for (int d = 0; d < dim; ++d) vr = vr + o.v[j * dim + d] * e[d];
                    double vij = (Zl * vl + Zr * vr + (o.p[i] - o.p[j])) / (Zl + Zr);
                    double ps = (Zl * o.p[j] + Zr * o.p[i] + Zl * Zr * (vl - vr)) / (Zl + Zr);
                    double vs[3];
                    for (int d = 0; d < dim; ++d)
                        vs[d] = vij * e[d] + ((o.v[i * dim + d] + o.v[j * dim + d]) / 2 - ((vl + vr) / 2) * e[d]);
                    double aux = 2 * ps * rhoij;
                    for (int d = 0; d < dim; ++d) {
                        double mm = 0;
                        for (int dd = 0; dd < dim; ++dd)
                            mm = mm + (o.visc[i] * E(i, d, dd) + o.visc[j] * E(j, d, dd)) * DW[k * dim + dd];
                        dvdt[d] = dvdt[d] + o.mass[j] * (-aux * DW[k * dim + d] + mm * rhoij);
                    }
                    double dot = 0;
                    for (int d = 0; d < dim; ++d) dot = dot + 2 * (o.v[i * dim + d] - vs[d]) * DW[k * dim + d];
                    dedt = dedt + o.mass[j] * aux * dot;
                }
            }
        } else {
            if (std::abs(o.type[i]) <= 100) {  // :230-251
                for (size_t k = 0; k < L.size(); ++k) {
                    int64_t j = L[k];
                    double aux = o.p[i] / (o.rho[i] * o.rho[i]) + o.p[j] / (o.rho[j] * o.rho[j]);
                    for (int d = 0; d < dim; ++d) {
                        double mm = 0;
                        for (int dd = 0; dd < dim; ++dd)
                            mm = mm + (o.visc[i] * E(i, d, dd) / (o.rho[i] * o.rho[i]) +
                                       (solid_j_dropped(o, j) ? 0.0 : o.visc[j] * E(j, d, dd) / (o.rho[j] * o.rho[j]))) *
                                          DW[k * dim + dd];
                        dvdt[d] = dvdt[d] + o.mass[j] * (-aux * DW[k * dim + d] + mm);
                    }
                    double dot = 0;
                    for (int d = 0; d < dim; ++d) dot = dot + (o.v[i * dim + d] - o.v[j * dim + d]) * DW[k * dim + d];
                    dedt = dedt + o.mass[j] * aux * dot;
                }
            } else {  // solid, :252-271
                for (size_t k = 0; k < L.size(); ++k) {
                    int64_t j = L[k];
                    for (int d = 0; d < dim; ++d) {
                        for (int dd = 0; dd < dim; ++dd)
                            dvdt[d] = dvdt[d] + o.mass[j] * (S(o.stress, i, d, dd) / (o.rho[i] * o.rho[i]) +
                                                            S(o.stress, j, d, dd) / (o.rho[j] * o.rho[j])) *
                                                    DW[k * dim + dd];
                        dedt = dedt + o.mass[j] * (o.p[i] / (o.rho[i] * o.rho[i]) + o.p[j] / (o.rho[j] * o.rho[j])) *
                                          (o.v[i * dim + d] - o.v[j * dim + d]) * DW[k * dim + d];
                    }
                }
            }
        }
        o.indedt[i] = o.tdsdt[i] + 0.5 * dedt;  // :332-334
    }
}

// ---- external force: src/Physic/externalForce.f90:7-175 ------------------
void external_force(Orc& o) {
    const int dim = o.dim;
    const sph_params& P = o.prm;
    const bool grav = P.flags & SPH_F_GRAVITY;
    const bool skip_solids = P.flags & SPH_F_GRAVITY_SKIP_SOLIDS;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < o.n_real; ++i) {
        double* a = &o.exdvdt[i * dim];
        for (int d = 0; d < dim; ++d) a[d] = 0;
        if (grav && !(skip_solids && o.type[i] > 100)) a[dim - 1] = P.gravity;
        double dx[3], dr, r;
        for (int32_t j : o.nl[i]) {
            if (o.type[i] > 0 && o.type[j] < 0) {  // real-dummy repulsion, :109-124
                dx[0] = o.x[i * dim] - o.x[(int64_t)j * dim];
                dr = dx[0] * dx[0];
                for (int d = 1; d < dim; ++d) { dx[d] = o.x[i * dim + d] - o.x[(int64_t)j * dim + d]; dr = dr + dx[d] * dx[d]; }
                r = std::sqrt(dr);
                if (r < P.wall_r0)
                    for (int d = 0; d < dim; ++d)
                        a[d] = a[d] + P.wall_fs * (std::pow(P.wall_r0 / r, P.wall_p1) - std::pow(P.wall_r0 / r, P.wall_p2)) * dx[d] / (r * r);
            }
            if (o.type[i] != o.type[j] && (o.type[i] > 0 && o.type[j] > 0)) {
                dx[0] = o.x[i * dim] - o.x[(int64_t)j * dim];
                dr = dx[0] * dx[0];
                for (int d = 1; d < dim; ++d) { dx[d] = o.x[i * dim + d] - o.x[(int64_t)j * dim + d]; dr = dr + dx[d] * dx[d]; }
                r = std::sqrt(dr);
                if (o.type[i] < 100 && o.type[j] < 100) {  // multiphase penalty, :127-141
                    double pe = (o.h[i] + o.h[j]) / (2 * r);
                    if (pe >= 1)
                        for (int d = 0; d < dim; ++d)
                            a[d] = a[d] + P.pen_factor * (std::pow(pe, P.pen_n1) - std::pow(pe, P.pen_n2)) * dx[d] / (r * r);
                } else if (!(o.type[i] > 100 && o.type[j] > 100)) {  // fluid-solid contact, :142-170
                    double eta = r / 0.75 / ((o.h[i] + o.h[j]) * 0.5);
                    double chi = 1 - r / P.contact_delta;
                    if (chi < 0 || chi > 1) chi = 0;
                    double fc;
                    if (eta <= 0 || eta >= 2) fc = 0;
                    else if (eta <= 2.0 / 3) fc = 2.0 / 3;
                    else if (eta <= 1) fc = 2 * eta - 1.5 * eta * eta;
                    else fc = 0.5 * ((2 - eta) * (2 - eta));
                    for (int d = 0; d < dim; ++d)
                        a[d] = a[d] + f32(0.01) * (o.c[i] * o.c[i]) * chi * fc * dx[d] / (r * r);
                }
            }
        }
    }
}

// ---- artificial viscosity: src/Numeric/artificialViscosity.f90:7-114 ------
void arti_visc(Orc& o) {
    const int dim = o.dim;
    const sph_params& P = o.prm;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < o.n_real; ++i) {
        double alpha = P.av_alpha, beta = P.av_beta, psi = P.av_psi;
        if (o.type[i] > 100) { alpha = P.av_alpha_solid; beta = P.av_beta_solid; }
        double* a = &o.avdvdt[i * dim];
        for (int d = 0; d < dim; ++d) a[d] = 0;
        double de = 0;
        const auto& L = o.nl[i];
        const double* DW = o.dwdx[i].data();
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            double dx[3], dv[3], xv = 0;
            for (int d = 0; d < dim; ++d) { dx[d] = o.x[i * dim + d] - o.x[j * dim + d]; dv[d] = o.v[i * dim + d] - o.v[j * dim + d]; }
            for (int d = 0; d < dim; ++d) xv = xv + dx[d] * dv[d];
            if (xv < 0.0) {
                double hij = 0.5 * (o.h[i] + o.h[j]);
                double rij = 0.5 * (o.rho[i] + o.rho[j]);
                double cij = 0.5 * (o.c[i] + o.c[j]);
                double s2 = 0;
                for (int d = 0; d < dim; ++d) s2 = s2 + dx[d] * dx[d];
                double phi = hij * xv / (s2 + (psi * hij) * (psi * hij));
                double PIij = (beta * phi - alpha * cij) * phi / rij;
                double aux[3], s = 0;
                for (int d = 0; d < dim; ++d) aux[d] = PIij * DW[k * dim + d];
                for (int d = 0; d < dim; ++d) a[d] = a[d] - o.mass[j] * aux[d];
                for (int d = 0; d < dim; ++d) s = s + dv[d] * aux[d];
                de = de + 0.5 * o.mass[j] * s;
            }
        }
        o.avdedt[i] = de;
    }
}

// ---- artificial heat: src/Numeric/artificialHeat.f90:6-56 ------------------
// q = alpha h c + beta h^2 (|div v| - div v) per particle (alpha 0.1, beta 1),
// pair averages of q, h and rho; dedt_i += 2 m_j aux (e_i - e_j) with
// aux = q_ij (dx . dW) / (rho_ij (r^2 + 0.01 h_ij^2)).  div v is this step's
// (divergence runs first, singleStep.f90:111); walls keep div v = 0.
void arti_heat(Orc& o) {
    const int dim = o.dim;
    const double alpha = 0.1, beta = 1.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < o.n_real; ++i) {
        double de = 0;
        const auto& L = o.nl[i];
        const double* DW = o.dwdx[i].data();
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            double qi = alpha * o.h[i] * o.c[i] + beta * (o.h[i] * o.h[i]) * (std::abs(o.divv[i]) - o.divv[i]);
            double qj = alpha * o.h[j] * o.c[j] + beta * (o.h[j] * o.h[j]) * (std::abs(o.divv[j]) - o.divv[j]);
            double qij = 0.5 * (qi + qj);
            double hij = 0.5 * (o.h[i] + o.h[j]);
            double rij = 0.5 * (o.rho[i] + o.rho[j]);
            double dx[3], s1 = 0, s2 = 0;
            for (int d = 0; d < dim; ++d) dx[d] = o.x[i * dim + d] - o.x[j * dim + d];
            for (int d = 0; d < dim; ++d) s1 = s1 + dx[d] * DW[k * dim + d];
            for (int d = 0; d < dim; ++d) s2 = s2 + dx[d] * dx[d];
            double aux = qij * s1 / (rij * (s2 + 0.01 * (hij * hij)));
            de = de + 2.0 * o.mass[j] * aux * (o.e[i] - o.e[j]);
        }
        o.ahdedt[i] = de;
    }
}

// ---- artificial stress: src/Numeric/artificialTerm.f90:7-98 (2-D) ---------
int artificial_stress(Orc& o) {
    const int dim = o.dim;
    const int64_t nt = o.n_real;
    for (int64_t i = 0; i < nt * dim; ++i) o.asdvdt[i] = 0;
    if (dim != 2) return SPH_E_UNSUPPORTED;  // error stop in the reference
    const double lambda = o.prm.as_eps, expo = o.prm.as_n, delta = o.prm.as_dp;
    std::vector<double> Rm(nt * 4, 0.0);
    auto ST = [&](int64_t i, int d, int dd) { return o.stress[i * 4 + dd * 2 + d]; };
    for (int64_t i = 0; i < nt; ++i) {
        if (o.type[i] < 100) continue;
        double aux = ST(i, 0, 0) - ST(i, 1, 1), theta;
        if (aux == 0) theta = 0.5 * PI;
        else theta = 0.5 * std::atan((ST(i, 0, 1) + ST(i, 1, 0)) / aux);
        double s = std::sin(theta), c = std::cos(theta);
        double ps[2], T[2];
        ps[0] = (c * c) * ST(i, 0, 0) + (s * s) * ST(i, 1, 1) + 2 * s * c * ST(i, 0, 1);
        ps[1] = (s * s) * ST(i, 0, 0) + (c * c) * ST(i, 1, 1) - 2 * s * c * ST(i, 0, 1);
        for (int d = 0; d < 2; ++d) T[d] = ps[d] > 0 ? -(lambda * ps[d] / (o.rho[i] * o.rho[i])) : 0.0;
        Rm[i * 4 + 0] = (c * c) * T[0] + (s * s) * T[1];
        Rm[i * 4 + 3] = (s * s) * T[0] + (c * c) * T[1];
        Rm[i * 4 + 2] = s * c * (T[0] - T[1]);
        Rm[i * 4 + 1] = Rm[i * 4 + 2];
    }
    for (int64_t i = 0; i < nt; ++i) {
        const auto& L = o.nl[i];
        double* a = &o.asdvdt[i * 2];
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            if (o.type[j] < 100) continue;
            double zero[2] = {0, 0}, tmp[2], wd;
            kernel(o.prm.skf, 2, delta, zero, o.h[i], wd, tmp);
            double F = std::pow(o.w[i][k] / wd, expo);
            for (int d = 0; d < 2; ++d)
                for (int e2 = 0; e2 < 2; ++e2) {
                    double Rj = j < nt ? Rm[j * 4 + e2 * 2 + d] : 0.0;
                    a[d] = a[d] + o.mass[j] * (Rm[i * 4 + e2 * 2 + d] + Rj) * F * o.dwdx[i][k * 2 + e2];
                }
        }
    }
    return SPH_OK;
}

// ---- XSPH: src/Numeric/correctVelocity.f90:7-44 ---------------------------
void aver_velo(Orc& o) {
    const int dim = o.dim;
    const double eps = o.prm.xsph_eps;
    for (int64_t i = 0; i < o.n_real; ++i) {
        double* a = &o.aver_v[i * dim];
        for (int d = 0; d < dim; ++d) a[d] = 0;
        if (o.boundary[i] == 1) continue;
        const auto& L = o.nl[i];
        for (size_t k = 0; k < L.size(); ++k) {
            int64_t j = L[k];
            for (int d = 0; d < dim; ++d) {
                double dv = o.v[i * dim + d] - o.v[j * dim + d];
                a[d] = a[d] - eps * 2 * o.mass[j] * dv / (o.rho[i] + o.rho[j]) * o.w[i][k];
            }
        }
    }
}

// ---- smoothing length: src/Numeric/hsml.f90:8-38 ---------------------------
void h_upgrade(Orc& o) {
    if (o.prm.sle == 1) {
        for (int64_t i = 0; i < o.n_real; ++i) o.h[i] = 2.0 * std::pow(o.mass[i] / o.rho[i], 1.0 / o.dim);
    } else if (o.prm.sle == 2) {
        for (int64_t i = 0; i < o.n_real; ++i) {
            double dh = (o.h[i] / o.dim) * o.divv[i];
            o.h[i] = o.h[i] + o.prm.dt * dh;
            if (o.h[i] <= 0) o.h[i] = o.h[i] - o.prm.dt * dh;
        }
    }
}

// ---- single_step: src/TimeIntegration/singleStep.f90:1-211 -----------------
int single_step(Orc& o) {
    const int dim = o.dim;
    const int64_t nt = o.n_real;
    const uint32_t F = o.prm.flags;
    o.indvdt.assign(nt * dim, 0.0); o.indedt.assign(nt, 0.0);
    o.exdvdt.assign(nt * dim, 0.0); o.avdvdt.assign(nt * dim, 0.0);
    o.avdedt.assign(nt, 0.0); o.asdvdt.assign(nt * dim, 0.0); o.ahdedt.assign(nt, 0.0);
    int st = bggs(o);  // :84
    if (st) return st;
    if (F & SPH_F_KERNEL_CORRECTION) kernel_correction(o);  // :86
    if (o.prm.pa_sph == 3) con_density_riemann(o);  // :98-99
    else if (F & SPH_F_SUM_DENSITY) sum_density(o);  // :91-105, SPH = 1/2
    else con_density(o);
    divergence(o);       // :111
    internal_force(o);   // :115
    bool exw = F & (SPH_F_EXT_FORCE | SPH_F_DUMMY | SPH_F_GRAVITY);  // getValueFromToml.f90:152-154
    if (exw) external_force(o);
    if (F & SPH_F_ARTI_VISC) arti_visc(o);
    if (F & SPH_F_ARTI_HEAT) arti_heat(o);  // :127
    if (F & SPH_F_ARTI_STRESS) { st = artificial_stress(o); if (st) return st; }
    if (F & SPH_F_AVER_VELOCITY) aver_velo(o);
    h_upgrade(o);
    for (int64_t i = 0; i < nt; ++i) {  // :139-142
        for (int d = 0; d < dim; ++d)
            o.dvdt[i * dim + d] = o.indvdt[i * dim + d] + o.avdvdt[i * dim + d] + o.exdvdt[i * dim + d] + o.asdvdt[i * dim + d];
        o.dedt[i] = o.indedt[i] + o.avdedt[i] + o.ahdedt[i];
    }
    for (int64_t i = 0; i < nt; ++i)  // fixedBoundary, boundaryCondition.f90:32-45
        if (o.boundary[i] == 1)
            for (int d = 0; d < dim; ++d) o.dvdt[i * dim + d] = 0;
    return SPH_OK;
}

// radial return of the deviatoric stress (timeIntegration.f90:145-167)
inline void yield_scale(const Orc& o, int64_t i, double* S) {
    const sph_material* m = material_of(o, o.type[i]);
    if (!m || !m->yield) return;
    const int D2 = o.dim * o.dim;
    double J2 = 0;
    for (int k = 0; k < D2; ++k) J2 = J2 + S[k] * S[k];
    double f = std::min(1.0, std::sqrt(((m->sigma_y * m->sigma_y) / 3) / J2));
    for (int k = 0; k < D2; ++k) S[k] = S[k] * f;
}
inline bool shear_type(int32_t t) { return t == 101 || t == 102 || t == 103 || t == 104; }

// courant_num, src/Numeric/courantNumber.f90:7-31
inline double courant(const Orc& o, double hs, double dvv, double c) {
    double a = o.prm.cour_alpha, b = o.prm.cour_beta;
    return o.prm.dt * (hs * dvv + c + f32(1.2) * (a * c + b * hs * std::abs(dvv))) / hs;
}

// One iteration of leap_frog's loop, timeIntegration.f90:85-263.
int leap_frog_step(Orc& o) {
    const int dim = o.dim, D2 = dim * dim;
    const int64_t nt = o.n_real;
    const double dt = o.prm.dt;
    const bool sumd = o.prm.flags & SPH_F_SUM_DENSITY;
    o.step += 1;
    if (o.step != 1) {  // half kick, :137-170
        for (int64_t i = 0; i < nt; ++i) {
            o.prev_e[i] = o.e[i];
            o.e[i] = o.e[i] + (dt / 2) * o.dedt[i];
            if (o.e[i] < 0) o.e[i] = 0;
            if (!sumd) { o.prev_rho[i] = o.rho[i]; o.rho[i] = o.rho[i] + (dt / 2) * o.drhodt[i]; }
            for (int d = 0; d < dim; ++d) {
                o.prev_v[i * dim + d] = o.v[i * dim + d];
                o.v[i * dim + d] = o.v[i * dim + d] + (dt / 2) * o.dvdt[i * dim + d];
            }
            if (shear_type(o.type[i])) {
                for (int k = 0; k < D2; ++k) {
                    o.shear_prev[i * D2 + k] = o.shear[i * D2 + k];
                    o.shear[i * D2 + k] = o.shear[i * D2 + k] + (dt / 2) * o.dsdt[i * D2 + k];
                }
                yield_scale(o, i, &o.shear[i * D2]);
            }
        }
    }
    int st = single_step(o);  // :172-176
    if (st) return st;
    if (o.step == 1) {  // :178-212
        for (int64_t i = 0; i < nt; ++i) {
            o.e[i] = o.e[i] + (dt / 2) * o.dedt[i];
            if (o.e[i] < 0) o.e[i] = 0;
            if (!sumd) o.rho[i] = o.rho[i] + (dt / 2) * o.drhodt[i];
            for (int d = 0; d < dim; ++d) {
                o.v[i * dim + d] = o.v[i * dim + d] + (dt / 2) * o.dvdt[i * dim + d] + o.aver_v[i * dim + d];
                o.disp[i * dim + d] = dt * o.v[i * dim + d];
                o.x[i * dim + d] = o.x[i * dim + d] + o.disp[i * dim + d];
            }
            if (shear_type(o.type[i])) {
                for (int k = 0; k < D2; ++k) o.shear[i * D2 + k] = o.shear[i * D2 + k] + (dt / 2) * o.dsdt[i * D2 + k];
                yield_scale(o, i, &o.shear[i * D2]);
            }
        }
    } else {  // :213-252
        double mx = 0, sum = 0;
        for (int64_t i = 0; i < nt; ++i) {
            o.e[i] = o.prev_e[i] + dt * o.dedt[i];
            if (o.e[i] < 0) o.e[i] = 0;
            if (!sumd) o.rho[i] = o.prev_rho[i] + dt * o.drhodt[i];
            for (int d = 0; d < dim; ++d) {
                o.v[i * dim + d] = o.prev_v[i * dim + d] + dt * o.dvdt[i * dim + d] + o.aver_v[i * dim + d];
                o.disp[i * dim + d] = o.disp[i * dim + d] + dt * o.v[i * dim + d];
                o.x[i * dim + d] = o.x[i * dim + d] + dt * o.v[i * dim + d];
            }
            if (shear_type(o.type[i])) {
                for (int k = 0; k < D2; ++k) o.shear[i * D2 + k] = o.shear_prev[i * D2 + k] + dt * o.dsdt[i * D2 + k];
                yield_scale(o, i, &o.shear[i * D2]);
            }
            double cn = courant(o, o.h[i], o.divv[i], o.c[i]);
            sum = sum + cn;
            if (cn > mx) mx = cn;
        }
        o.max_courant = mx;
        // aver_courant is not reset before the reduction in the reference
        // (timeIntegration.f90:213-251), so the previous mean carries over.
        o.aver_courant = (o.aver_courant + sum) / nt;
    }
    o.time = o.time + dt;
    return SPH_OK;
}

}  // namespace

// ============================ C API (ctypes) ==============================
extern "C" {

typedef struct Orc orc_t;

#define ORC_FIELD_IN_DVDT  101
#define ORC_FIELD_IN_DEDT  102
#define ORC_FIELD_EX_DVDT  103
#define ORC_FIELD_AV_DVDT  104
#define ORC_FIELD_AV_DEDT  105
#define ORC_FIELD_AS_DVDT  106
#define ORC_FIELD_TDSDT    107
#define ORC_FIELD_ROT      108
#define ORC_FIELD_AH_DEDT  109

int orc_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

void* orc_create(const sph_params* prm, int64_t n_real, int64_t n_wall,
                 const double* x, const double* v, const double* mass, const double* rho,
                 const double* p, const double* e, const double* c, const double* h,
                 const int32_t* type, const int32_t* state, const int32_t* boundary,
                 const double* shear) {
    if (!prm || prm->dim < 1 || prm->dim > 3 || n_real <= 0 || n_wall < 0) return nullptr;
    Orc* o = new Orc();
    o->prm = *prm;
    o->dim = prm->dim;
    o->n_real = n_real; o->n_wall = n_wall; o->N = n_real + n_wall;
    const int64_t N = o->N, dim = o->dim, D2 = dim * dim;
    o->x.assign(x, x + N * dim);
    o->v.assign(v, v + N * dim);
    o->disp.assign(N * dim, 0.0);
    o->mass.assign(mass, mass + N); o->rho.assign(rho, rho + N);
    o->p.assign(p, p + N); o->e.assign(e, e + N);
    o->c.assign(c, c + N); o->h.assign(h, h + N);
    o->visc.assign(N, 0.0); o->divx.assign(N, 0.0); o->divv.assign(N, 0.0);
    o->type.assign(type, type + N);
    if (state) o->state.assign(state, state + N); else o->state.assign(N, 0);
    if (boundary) o->boundary.assign(boundary, boundary + N); else o->boundary.assign(N, 0);
    o->stress.assign(N * D2, 0.0);
    if (shear) o->shear.assign(shear, shear + N * D2); else o->shear.assign(N * D2, 0.0);
    o->shear_prev.assign(N * D2, 0.0); o->dsdt.assign(N * D2, 0.0);
    o->prev_v.assign(N * dim, 0.0); o->prev_rho.assign(N, 0.0); o->prev_e.assign(N, 0.0);
    o->dvdt.assign(N * dim, 0.0); o->drhodt.assign(N, 0.0); o->dedt.assign(N, 0.0);
    o->aver_v.assign(N * dim, 0.0);
    return o;
}

void orc_destroy(void* h) { delete (Orc*)h; }

int orc_bggs(void* h) { return bggs(*(Orc*)h); }

int orc_set_search(void* h, int32_t mode) {
    ((Orc*)h)->search_mode = mode;
    return SPH_OK;
}

int64_t orc_neighbor_total(void* h) {
    Orc& o = *(Orc*)h;
    int64_t t = 0;
    for (auto& l : o.nl) t += (int64_t)l.size();
    return t;
}

// Lists in the reference's order, 1-based source indices.
int orc_export_neighbors(void* h, int64_t* offsets, int32_t* list, int64_t cap) {
    Orc& o = *(Orc*)h;
    int64_t t = 0;
    offsets[0] = 0;
    for (int64_t i = 0; i < o.n_real; ++i) {
        const auto& l = i < (int64_t)o.nl.size() ? o.nl[i] : std::vector<int32_t>();
        if (t + (int64_t)l.size() > cap) return SPH_E_OVERFLOW;
        for (int32_t j : l) list[t++] = j + 1;
        offsets[i + 1] = t;
    }
    return SPH_OK;
}

// Rates of one single_step without advancing time (parity of the modules).
int orc_rates(void* h) { return single_step(*(Orc*)h); }

int orc_single_step(void* h) { return leap_frog_step(*(Orc*)h); }

int orc_advance(void* h, int64_t nsteps, double* maxc, double* meanc) {
    Orc& o = *(Orc*)h;
    for (int64_t s = 0; s < nsteps; ++s) {
        int st = leap_frog_step(o);
        if (st) return st;
    }
    if (maxc) *maxc = o.max_courant;
    if (meanc) *meanc = o.aver_courant;
    return SPH_OK;
}

int orc_info(void* h, int64_t* step, double* time) {
    Orc& o = *(Orc*)h;
    if (step) *step = o.step;
    if (time) *time = o.time;
    return SPH_OK;
}

// Copy a field of all N particles (module outputs: n_real entries).
int orc_get_field(void* h, int32_t field, double* out) {
    Orc& o = *(Orc*)h;
    const int64_t N = o.N, nt = o.n_real, dim = o.dim, D2 = dim * dim;
    auto cp = [&](const std::vector<double>& a, int64_t n) {
        if ((int64_t)a.size() < n) return SPH_E_STATE;
        std::memcpy(out, a.data(), n * sizeof(double));
        return SPH_OK;
    };
    switch (field) {
    case SPH_FIELD_X: return cp(o.x, N * dim);
    case SPH_FIELD_V: return cp(o.v, N * dim);
    case SPH_FIELD_MASS: return cp(o.mass, N);
    case SPH_FIELD_RHO: return cp(o.rho, N);
    case SPH_FIELD_P: return cp(o.p, N);
    case SPH_FIELD_E: return cp(o.e, N);
    case SPH_FIELD_C: return cp(o.c, N);
    case SPH_FIELD_H: return cp(o.h, N);
    case SPH_FIELD_DIVX: return cp(o.divx, N);
    case SPH_FIELD_DIVV: return cp(o.divv, N);
    case SPH_FIELD_DISP: return cp(o.disp, N * dim);
    case SPH_FIELD_STRESS: return cp(o.stress, N * D2);
    case SPH_FIELD_SHEAR: return cp(o.shear, N * D2);
    case SPH_FIELD_DSDT: return cp(o.dsdt, N * D2);
    case SPH_FIELD_DVDT: return cp(o.dvdt, N * dim);
    case SPH_FIELD_DRHODT: return cp(o.drhodt, N);
    case SPH_FIELD_DEDT: return cp(o.dedt, N);
    case SPH_FIELD_VISC: return cp(o.visc, N);
    case SPH_FIELD_STRAIN: return cp(o.edot, N * D2);
    case SPH_FIELD_AVER: return cp(o.aver_v, N * dim);
    case SPH_FIELD_NNEIGH:
        for (int64_t i = 0; i < N; ++i) out[i] = i < (int64_t)o.nl.size() ? (double)o.nl[i].size() : 0.0;
        return SPH_OK;
    case SPH_FIELD_TYPE:
        for (int64_t i = 0; i < N; ++i) out[i] = o.type[i];
        return SPH_OK;
    case ORC_FIELD_IN_DVDT: return cp(o.indvdt, nt * dim);
    case ORC_FIELD_IN_DEDT: return cp(o.indedt, nt);
    case ORC_FIELD_EX_DVDT: return cp(o.exdvdt, nt * dim);
    case ORC_FIELD_AV_DVDT: return cp(o.avdvdt, nt * dim);
    case ORC_FIELD_AV_DEDT: return cp(o.avdedt, nt);
    case ORC_FIELD_AS_DVDT: return cp(o.asdvdt, nt * dim);
    case ORC_FIELD_TDSDT: return cp(o.tdsdt, N);
    case ORC_FIELD_ROT: return cp(o.rdot, N * D2);
    case ORC_FIELD_AH_DEDT: return cp(o.ahdedt, nt);
    default: return SPH_E_INVALID;
    }
}

// Evaluate the kernel (known-answer tests of kernel.f90).
int orc_kernel(int32_t skf, int32_t dim, double r, const double* dx, double hsml, double* w, double* dwdx) {
    double ww = 0;
    kernel(skf, dim, r, dx, hsml, ww, dwdx);
    *w = ww;
    return SPH_OK;
}

// Evaluate the EOS of a material (known-answer tests of eos.f90).
int orc_eos(const sph_material* m, int32_t solid, double rho, double e, double* p, double* c) {
    if (solid) solid_eos(m, rho, e, *p);
    else fluid_eos(m, rho, e, *p, *c);
    return SPH_OK;
}

}  // extern "C"
