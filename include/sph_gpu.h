/*
 * sph_gpu.h — C ABI of libsphgpu.so, the GB300 (sm_103a) per-step particle
 * hot path of the mySPH solver (SZWHTQ/mySPH).
 *
 * Everything here is plain C: fixed-width integers, doubles, pointers and
 * sizes.  No C++ or CUDA types cross the boundary, so the Fortran host can
 * bind every entry point with `iso_c_binding` (a `bind(C)` interface module) and
 * Python with ctypes.
 *
 * Conventions (they replace the reference's own, which are listed beside):
 *  - ownership: the caller owns every host array; the library copies in
 *    (sph_upload) and out (sph_download / sph_get_field).  Device state lives
 *    in the context between calls.  The reference mutates `type(Particle)`
 *    arrays in place (src/TimeIntegration/singleStep.f90:1-35).
 *  - layout: Fortran column-major.  Vector fields are X(Dim,N), element
 *    (d,n) at x[n*dim + d]; tensor fields are S(Dim,Dim,N), element
 *    (d,dd,n) at s[n*dim*dim + dd*dim + d].  Particles 0..n_real-1 are the
 *    real (fluid/solid) particles, n_real..n_real+n_wall-1 the wall ("dummy")
 *    particles, exactly as the reference stores dummies after ntotal
 *    (src/Physic/dummyParticles.f90:9-45).  Neighbour indices exported by
 *    sph_export_neighbors are 1-based like the reference's neighborList.
 *  - errors: every entry point returns an int status, 0 = SPH_OK, < 0 an
 *    SPH_E_* code; nothing aborts the process.  The reference calls
 *    `error stop` instead (src/NNPS/asymmetricSearch.f90:38-39,
 *    src/TimeIntegration/singleStep.f90:102-104).
 *  - threading: one context per host thread; all work of a context is
 *    ordered on its CUDA stream.  There is no global mutable state: the
 *    reference's `save` variables (src/Physic/externalForce.f90:13-16) are
 *    context fields (sph_params).
 */
#ifndef SPH_GPU_H
#define SPH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define SPH_OK               0
#define SPH_E_INVALID      (-1)  /* bad argument (null pointer, size, dim)   */
#define SPH_E_NOMEM        (-2)  /* device allocation failed / over budget   */
#define SPH_E_CUDA         (-3)  /* a CUDA runtime call failed               */
#define SPH_E_STATE        (-4)  /* call out of order (e.g. step before upload) */
#define SPH_E_UNSUPPORTED  (-5)  /* option not implemented on the GPU path   */
#define SPH_E_NONFINITE    (-6)  /* NaN/Inf detected in rho/v/e by a kernel  */
#define SPH_E_OVERFLOW     (-7)  /* neighbour count above the export buffer  */
#define SPH_E_TIMEOUT      (-8)  /* a bounded device wait gave up            */
#define SPH_E_RANGE        (-9)  /* a particle left the hash domain (clamped,
                                    reported as a warning bit only)          */
#define SPH_E_TOO_LARGE   (-10)  /* input larger than the fixed scratch of an
                                    allocation-free entry point              */

/* ---- configuration flags (sph.toml [Parameter] switches) ---------------- *
 * src/Initialize/getValueFromToml.f90:135-154 */
#define SPH_F_SUM_DENSITY      (1u << 0)  /* summationDensity                 */
#define SPH_F_NORM_DENSITY     (1u << 1)  /* normalizeDensity                 */
#define SPH_F_VISCOSITY        (1u << 2)  /* viscosity                        */
#define SPH_F_GRAVITY          (1u << 3)  /* gravity                          */
#define SPH_F_EXT_FORCE        (1u << 4)  /* externalForce (forced on by dummyParticle/gravity) */
#define SPH_F_ARTI_VISC        (1u << 5)  /* artificialViscosity              */
#define SPH_F_ARTI_STRESS      (1u << 6)  /* artificialStress                 */
#define SPH_F_AVER_VELOCITY    (1u << 7)  /* averageVelocity (XSPH)           */
#define SPH_F_DUMMY            (1u << 8)  /* dummyParticle                    */
/* nick-keyed behaviours of the reference, made explicit: */
#define SPH_F_GRAVITY_SKIP_SOLIDS (1u << 9)  /* Type>100 gets no gravity:
                                               externalForce.f90:42-48 (db_gate, water_impact) */
/* A fix, off by default: in the fluid branch of internal_force a solid
 * neighbour j contributes no viscous term.  The reference adds
 * Viscosity(j)*edot(j) for every neighbour (internalForce.f90:242-243), and
 * for a solid Viscosity is the shear modulus (viscosity.f90:21-28), which
 * makes fluid-structure runs unstable at any practical time step. */
#define SPH_F_FSI_FLUID_VISCOUS   (1u << 10)
/* kernelCorrection (kernelGradientCorrection.f90:8-51): every neighbour
 * gradient of a target becomes the solution x of A_i x = dW_ij, with
 * A_i = sum_j (x_j - x_i) (x) dW_ij m_j/rho_j over neighbours whose
 * (|Type|-100) has the target's sign, solved by the reference's pivoted
 * elimination (tools.f90:287-354).  FP64 path only; every real particle
 * must be a solid (Type > 100): for other targets A_i is zero and the
 * reference's solve divides 0 by 0. */
#define SPH_F_KERNEL_CORRECTION   (1u << 11)
/* artificialHeat (artificialHeat.f90:6-56): the heat-conduction term
 * de_i += 2 m_j q_ij (x_ij . dW_ij) (e_i - e_j) / (rho_ij (r^2 + 0.01 h_ij^2))
 * with q = 0.1 h c + h^2 (|div v| - div v) per particle and pair averages;
 * added to the energy rate after the artificial viscosity
 * (singleStep.f90:127, 141).  FP64 path with SPH = 2, without kernel
 * correction. */
#define SPH_F_ARTI_HEAT           (1u << 12)

/* ---- equation-of-state kinds (src/Physic/eos.f90) ----------------------- */
#define SPH_EOS_NONE        0
#define SPH_EOS_GAS         1   /* gamma law, eos.f90:9-18                   */
#define SPH_EOS_TAIT        2   /* arti_water_eos_1, eos.f90:23-53           */
#define SPH_EOS_MORRIS      3   /* arti_water_eos_2, eos.f90:57-64           */
#define SPH_EOS_MG_SOLID    101 /* Mie-Gruneisen solid, eos.f90:180-215      */
#define SPH_EOS_LINEAR      102 /* p = K/rho0 (rho-rho0), eos.f90:219-248    */

#define SPH_MAX_MATERIALS   8

/* One row of the material table.  It replaces the reference's per-|Type|
 * hard-coded constants: EOS (src/Physic/eos.f90), viscosity / shear modulus
 * (src/Physic/viscosity.f90:5-35) and yield stress of the J2 radial return
 * (src/TimeIntegration/timeIntegration.f90:147-158). */
typedef struct sph_material {
    int32_t type;     /* |Type| this row applies to (2, 101, 102, ...)        */
    int32_t eos;      /* SPH_EOS_*                                            */
    int32_t solid;    /* 1: solid branch (Type > 100 in the reference)        */
    int32_t yield;    /* 1: J2 radial return with sigma_y after each update    */
    double  rho0;     /* reference density                                    */
    double  c0;       /* Tait sound speed (B = c0^2 rho0 / gamma)             */
    double  gamma;    /* Tait / gas exponent, Mie-Gruneisen Gamma             */
    double  K;        /* linear solid bulk modulus (p = K/rho0 (rho-rho0))    */
    double  eta;      /* fluid dynamic viscosity or solid shear modulus G     */
    double  sigma_y;  /* yield stress                                         */
    double  mg_cs;    /* Mie-Gruneisen Hugoniot Cs                            */
    double  mg_s;     /* Mie-Gruneisen Hugoniot S                             */
} sph_material;

/* Precision of the pair loops. */
#define SPH_PREC_FP64   0   /* plain: every per-particle and pair operation in FP64 */
#define SPH_PREC_MIXED  1   /* FP32 kernel weights / EOS / pair forces with
                               compensated sums; FP64 positions, integration,
                               dt and energy reductions                         */
#define SPH_PREC_DF64   2   /* pair physics in double-float arithmetic (pairs of
                               FP32, about 48 significant bits) on the FP32
                               pipes; the neighbour test, per-particle epilogues
                               and the update in FP64.  Fluid systems with the
                               cubic spline, without kernel correction or
                               artificial stress.                               */

/* Run parameters: the sph.toml keys of src/Initialize/getValueFromToml.f90:95-185
 * plus every constant the reference hard-codes per case nick. */
typedef struct sph_params {
    int32_t  dim;          /* DIM: 2 or 3 on the GPU (the oracle also takes 1) */
    int32_t  skf;          /* SKF: 1 cubic spline, 2 Gauss, 3 quintic          */
    int32_t  pa_sph;       /* SPH (internalForce.f90:194-329): 2 P/rho^2 form;
                              1 (P_i+P_j)/(rho_i rho_j) form; 3 PVRS Riemann
                              solver, with con_density_riemann for the density.
                              1 and 3 in SPH_PREC_FP64 without kernel
                              correction; solid targets get no internal force
                              under them, as in the reference                  */
    int32_t  sle;          /* SLE (hsml.f90:8-38): 0 constant h; 1 h = 2 (m/rho)^(1/dim);
                              2 dh/dt = h/dim div v.  With 1 or 2 set cell_size to
                              scale_k times the largest h expected: an h beyond it
                              ends the step with SPH_E_RANGE                    */
    uint32_t flags;        /* SPH_F_*                                          */
    int32_t  precision;    /* SPH_PREC_*                                       */
    double   dt;           /* deltaT (fixed step)                              */

    /* gravity (externalForce.f90:27-59): acceleration on axis dim-1 */
    double   gravity;      /* -9.81 in the reference                           */

    /* Monaghan artificial viscosity (per-nick alpha, beta, psi: artificialViscosity.f90:30-79) */
    double   av_alpha, av_beta, av_psi;
    double   av_alpha_solid, av_beta_solid;   /* Type>100 override         */

    /* Courant number coefficients (courantNumber.f90:12-25) */
    double   cour_alpha, cour_beta;

    /* wall repulsion, multiphase penalty, fluid-solid contact
       (externalForce.f90:62-101) */
    double   wall_fs, wall_r0, wall_p1, wall_p2;
    double   pen_factor, pen_n1, pen_n2;
    double   contact_delta;

    /* artificial stress (artificialTerm.f90:17-32) */
    double   as_eps, as_n, as_dp;

    /* XSPH epsilon (correctVelocity.f90:20) */
    double   xsph_eps;

    /* material table */
    int32_t  n_materials;
    int32_t  reserved0;
    sph_material materials[SPH_MAX_MATERIALS];

    /* hash grid (GPU only).  cell_size <= 0: scale_k * max h.  If
       domain_lo >= domain_hi on any axis the grid domain is the bounding box
       of the uploaded particles grown by grid_margin on every side.
       Particles outside the domain are clamped into the border cells, which
       keeps the neighbour search exact. */
    double   cell_size;
    double   domain_lo[3], domain_hi[3];
    double   grid_margin;
} sph_params;

/* ---- field identifiers for sph_get_field / sph_set_field ---------------- */
#define SPH_FIELD_X           1   /* Dim per particle                       */
#define SPH_FIELD_V           2   /* Dim                                    */
#define SPH_FIELD_MASS        3
#define SPH_FIELD_RHO         4
#define SPH_FIELD_P           5
#define SPH_FIELD_E           6
#define SPH_FIELD_C           7
#define SPH_FIELD_H           8
#define SPH_FIELD_DIVX        9   /* divergencePosition                     */
#define SPH_FIELD_DIVV        10  /* divergenceVelocity                     */
#define SPH_FIELD_DISP        11  /* Displacement, Dim                      */
#define SPH_FIELD_STRESS      12  /* Stress, Dim*Dim                        */
#define SPH_FIELD_SHEAR       13  /* deviatoric stress, Dim*Dim             */
#define SPH_FIELD_DSDT        14  /* Dim*Dim                                */
#define SPH_FIELD_DVDT        15  /* Delta%Velocity, Dim                    */
#define SPH_FIELD_DRHODT      16  /* Delta%Density                          */
#define SPH_FIELD_DEDT        17  /* Delta%Energy                           */
#define SPH_FIELD_NNEIGH      18  /* neighbour count (as double)            */
#define SPH_FIELD_TYPE        19  /* Type (as double)                       */
#define SPH_FIELD_VISC        20  /* Viscosity (eta or G)                   */
#define SPH_FIELD_STRAIN      21  /* edot, Dim*Dim                          */
#define SPH_FIELD_AVER        22  /* aver_v, the XSPH velocity correction   */
                                  /* (correctVelocity.f90:7-44), Dim        */

/* force terms for the per-module parity calls */
#define SPH_TERM_INTERNAL     (1u << 0)
#define SPH_TERM_ARTI_VISC    (1u << 1)
#define SPH_TERM_EXTERNAL     (1u << 2)
#define SPH_TERM_ARTI_STRESS  (1u << 3)
#define SPH_TERM_ARTI_HEAT    (1u << 4)
#define SPH_TERM_ALL          0x1Fu

typedef struct sph_ctx sph_ctx;

/* ---- lifecycle ---------------------------------------------------------- */

/* Library ABI version (SPH_ABI_VERSION). */
int sph_abi_version(void);

/* Fill *prm with the defaults of getValueFromToml.f90:113-151 and the
 * reference's `case default` constants (water material type 2). */
int sph_params_default(sph_params* prm);

/* Create a context for up to `capacity` particles (real + wall) on the
 * current CUDA device.  Replaces allocateParticleList
 * (src/Initialize/SPH.f90:126-136) and the leap-frog arrays of
 * src/TimeIntegration/timeIntegration.f90:38-66. */
int sph_create(const sph_params* prm, int64_t capacity, sph_ctx** out);
int sph_destroy(sph_ctx* ctx);

/* Replace the run parameters (dt, flags, constants) of a context. */
int sph_set_params(sph_ctx* ctx, const sph_params* prm);

/* Upload a full particle set (host arrays, layout above).  `shear` may be
 * NULL (zero deviatoric stress).  Resets the leap-frog step counter, so the
 * next step is a "first step" (timeIntegration.f90:178-212).  Replaces
 * input()/write_initial_file (src/Initialize/input.f90:9-19) as the entry
 * of particle data. */
int sph_upload(sph_ctx* ctx, int64_t n_real, int64_t n_wall,
               const double* x, const double* v, const double* mass,
               const double* rho, const double* p, const double* e,
               const double* c, const double* h, const int32_t* type,
               const int32_t* state, const int32_t* boundary,
               const double* shear);

/* Copy the evolving state back (any pointer may be NULL to skip that
 * field).  Arrays are in the uploaded particle order and cover real and
 * wall particles (n_real + n_wall entries). */
int sph_download(sph_ctx* ctx, double* x, double* v, double* rho, double* p,
                 double* e, double* c, double* shear);

/* Copy one field (SPH_FIELD_*) of all n_real + n_wall particles, in the
 * uploaded order, into `out` (count = components * (n_real + n_wall)). */
int sph_get_field(sph_ctx* ctx, int32_t field, double* out);

/* Overwrite one field of all particles from a host array (SPH_FIELD_X, V,
 * RHO, P, E, C, H, MASS, SHEAR, DVDT, DRHODT, DEDT, DSDT, DIVX). */
int sph_set_field(sph_ctx* ctx, int32_t field, const double* in);

/* Particle counts, step counter and simulated time. */
int sph_info(sph_ctx* ctx, int64_t* n_real, int64_t* n_wall, int64_t* step,
             double* time);

/* ---- per-module parity entry points ------------------------------------ *
 * Each runs on the device on the current state and writes its result to
 * host arrays (n_real entries, uploaded order).  They mirror the module
 * procedures of the reference one by one. */

/* Build the cell hash (keys, radix sort, cell ranges) over all particles.
 * Replaces BGGS's grid (src/NNPS/asymmetricSearch.f90:49-158). */
int sph_nnps(sph_ctx* ctx);

/* Number of neighbours of every real particle and their sum, after
 * sph_nnps.  `counts` may be NULL.  Same sets as BGGS
 * (asymmetricSearch.f90:160-257): j != i, State_j != -1, r < scale_k*h_i. */
int sph_neighbor_counts(sph_ctx* ctx, int32_t* counts, int64_t* total);

/* Export the neighbour lists in CSR form: offsets[n_real+1], list[total]
 * with 1-based uploaded indices; `capacity` is the size of `list`.  The
 * GPU never stores these lists on the step path; this is a test export. */
int sph_export_neighbors(sph_ctx* ctx, int64_t* offsets, int32_t* list,
                         int64_t capacity);

/* con_density (src/Physic/density.f90:83-107) -> drhodt[n_real].
 * With SPH_F_SUM_DENSITY, sum_density (density.f90:10-80) instead: the
 * density of every real particle becomes m_i W(0,h_i) + sum_j m_j W_ij,
 * divided by m_i/rho_i W(0,h_i) + sum_j m_j/rho_j W_ij where
 * SPH_F_NORM_DENSITY is set and the particle's divergencePosition of the
 * previous step is below 1.5; drhodt (may be NULL) receives zeros.  Like
 * single_step, a context runs sum_density once per neighbour search: every
 * module call after sph_nnps sees the summed density. */
int sph_density(sph_ctx* ctx, double* drhodt);

/* divergence (src/Numeric/divergence.f90:6-29). */
int sph_divergence(sph_ctx* ctx, double* div_x, double* div_v);

/* internal_force (src/Physic/internalForce.f90:10-342): EOS of every
 * particle, strain rates, deviatoric stress rate and the momentum/energy
 * pair sums.  dvdt[n_real*dim], dedt[n_real]; dsdt may be NULL. */
int sph_internal_force(sph_ctx* ctx, double* dvdt, double* dedt, double* dsdt);

/* external_force (src/Physic/externalForce.f90:7-175). */
int sph_external_force(sph_ctx* ctx, double* dvdt);

/* arti_visc (src/Numeric/artificialViscosity.f90:7-114). */
int sph_arti_visc(sph_ctx* ctx, double* dvdt, double* dedt);

/* artificialStress (src/Numeric/artificialTerm.f90:7-98), 2-D only. */
int sph_arti_stress(sph_ctx* ctx, double* dvdt);
/* arti_heat(ntotal, P, dedt) (artificialHeat.f90:6-56): the artificial-heat
 * energy rate of every real particle (needs SPH_F_ARTI_HEAT's model: FP64,
 * SPH = 2, no kernel correction). */
int sph_arti_heat(sph_ctx* ctx, double* dedt);

/* single_step's assembled rates after boundary()
 * (src/TimeIntegration/singleStep.f90:139-144,
 *  src/Physic/boundaryCondition.f90:32-45): Delta%Velocity, Delta%Density,
 * Delta%Energy.  Does not advance time. */
int sph_rates(sph_ctx* ctx, double* dvdt, double* drhodt, double* dedt);

/* ---- performance entry points ------------------------------------------ */

/* One iteration of leap_frog's loop (timeIntegration.f90:85-263 without
 * output): half-kick, single_step, full update, Courant statistics. */
int sph_single_step(sph_ctx* ctx);

/* `nsteps` iterations without returning to the host in between.
 * max_courant / mean_courant (may be NULL) receive the statistics of the
 * last step (timeIntegration.f90:213-252). */
int sph_advance(sph_ctx* ctx, int64_t nsteps, double* max_courant,
                double* mean_courant);

/* sph_advance split in two, so that one host thread can keep several
 * contexts busy at once: sph_advance_async queues `nsteps` iterations on the
 * context's own stream and returns without waiting for them; sph_sync waits
 * for the context's queued work and returns what sph_advance would have
 * returned for it (SPH_E_NONFINITE and the other step errors surface here),
 * with the Courant statistics of the last step (pointers may be NULL).
 * Contexts have separate streams, so the steps of two contexts queued back
 * to back run concurrently on the device.  No other call may be made on the
 * context between the two, except further sph_advance_async calls. */
int sph_advance_async(sph_ctx* ctx, int64_t nsteps);
int sph_sync(sph_ctx* ctx, double* max_courant, double* mean_courant);

/* The drop-in form of leap_frog's loop for a host that owns the particle
 * arrays (the reference's P(:), timeIntegration.f90:32-285): copy the real
 * particles' x, v, rho, e (and shear, may be NULL) in from host memory, run
 * `nsteps` iterations on the device and copy the same arrays back, in the
 * uploaded order (n_real entries; x, v: dim per particle; shear: dim*dim).
 * The leap-frog Prev/Delta arrays stay on the device between calls, as they
 * live inside leap_frog in the reference.  Host buffers may be pinned. */
int sph_step_host(sph_ctx* ctx, int64_t nsteps, double* x, double* v, double* rho,
                  double* e, double* shear);

/* Energy sums of the real particles in FP64, summed in a fixed order (the
 * same bits on every call for the same state): out[0] kinetic
 * sum 1/2 m v.v, out[1] internal sum m e, out[2] gravitational
 * sum -m g x_(dim-1) (0 without SPH_F_GRAVITY), out[3] their total.  On a
 * batch context `inst` selects one system (or -1 for all); a plain context
 * ignores it.  The reference keeps no such sum; it is the diagnostic of the
 * mixed-precision form, whose energy bookkeeping stays FP64. */
int sph_energy(sph_ctx* ctx, int32_t inst, double out[4]);

/* Neighbour statistics of the last search (src/NNPS/nnps.f90:377-416):
 * out[0] max, out[1] min, out[2] mean, out[3] #particles without
 * neighbours, out[4] 1-based index of the max, out[5] of the min. */
int sph_statistics(sph_ctx* ctx, double out[6]);

/* boundary (boundaryCondition.f90:15-45) after per-module calls: its
 * fixedBoundary zeroes the velocity rate of every particle with Boundary == 1,
 * in dvdt (host, n_real x dim in upload order, in/out, may be NULL) and in the
 * context's assembled rates.  The nick-specific sponge layer and prescribed
 * displacement of boundary() are not part of this path.  Plain contexts. */
int sph_boundary(sph_ctx* ctx, double* dvdt);

/* courant_num (courantNumber.f90:7-31), elementwise, on the device with the
 * context's deltaT and Courant alpha / beta:
 *   xi = dt (h div_v + c + 1.2 (alpha c + beta h |div_v|)) / h
 * (1.2 the single-precision literal).  Host arrays of n values. */
int sph_courant_num(sph_ctx* ctx, int64_t n, const double* hsml, const double* div_v, const double* c,
                    double* xi);

/* ---- batches of independent particle systems ---------------------------- *
 * No counterpart in the reference, which runs one case per process.  A batch
 * advances many independent systems ("instances") together: one launch per
 * stage covers all of them, each with its own hash grid, material table and
 * time step (sph_params.dt of its sph_batch_add).  All instances share the
 * model of the batch (dim, kernel, flags, AV, wall force, ...); sph_batch_add
 * rejects a different one.  sph_advance / sph_single_step step every live
 * instance; an instance added later takes its own first (no-kick) step.  */

/* A batch with room for `max_instances` systems, `real_capacity` real and
 * `wall_capacity` wall particles in total (all device memory is reserved
 * here, so admission never allocates particle storage). */
int sph_batch_create(const sph_params* prm, int32_t max_instances, int64_t real_capacity,
                     int64_t wall_capacity, sph_ctx** out);

/* Add one system (arrays as sph_upload, its n_real + n_wall particles in its
 * own order).  *inst receives its slot.  SPH_E_NOMEM when the batch is full. */
int sph_batch_add(sph_ctx* ctx, const sph_params* prm, int64_t n_real, int64_t n_wall,
                  const double* x, const double* v, const double* mass, const double* rho,
                  const double* p, const double* e, const double* c, const double* h,
                  const int32_t* type, const int32_t* state, const int32_t* boundary,
                  const double* shear, int32_t* inst);

/* ---- device-side case generation ----------------------------------------- *
 * The reference's case generators (input.f90:1031-1405 and the wall layers of
 * dummyParticles.f90:544-765) build their particles from lattice blocks.  A
 * block is generated on the device, so a case of any size is described by a
 * few hundred bytes instead of uploaded particle arrays.  Particle (i, j, k)
 * of a block (index (i n[1] + j) n[2] + k) sits at
 *   x_a = origin_a + (i_a + 1/2) spacing_a
 * (spacing 0 with n = 1 gives a constant coordinate) and gets:
 *   mass, h, c, type, state of the block;
 *   p = p_rho0_g * max(p_level - x_up, 0)            (0 when p_rho0_g == 0)
 *   rho = tait_rho0 (p / tait_b + 1)^(1 / tait_gamma) (when tait_b > 0; the
 *         inverse Tait EOS, eos.f90:43-47), else rho;
 *   v_a = v_a + v_ramp_a max(x_0, 0) / v_ramp_len   (v_ramp_len > 0);
 *   Boundary = 1 and v = 0 where x_c < clamp_below or x_c > clamp_above,
 *   c = clamp_axis (fixedBoundary rows, e.g. a clamped root or top edge).
 * The first n_real_blocks blocks are real particles, the rest walls. */
typedef struct sph_block {
    int32_t n[3];
    int32_t type, state, up_axis;
    int32_t clamp_axis, reserved;
    double origin[3], spacing[3];
    double mass, h, c, rho;
    double p_rho0_g, p_level;
    double tait_b, tait_gamma, tait_rho0;
    double v[3], v_ramp[3], v_ramp_len;
    double clamp_below, clamp_above;
} sph_block;

/* Replace the particles of a plain context by generated blocks (as
 * sph_upload). */
int sph_upload_blocks(sph_ctx* ctx, int32_t n_blocks, const sph_block* blocks,
                      int32_t n_real_blocks);

/* Add a system built from generated blocks to a batch (as sph_batch_add). */
int sph_batch_add_blocks(sph_ctx* ctx, const sph_params* prm, int32_t n_blocks,
                         const sph_block* blocks, int32_t n_real_blocks, int32_t* inst);

/* Retire a system: its particles leave at the next step, its slot is free. */
int sph_batch_remove(sph_ctx* ctx, int32_t inst);

/* One field of one system, in the order of its sph_batch_add arrays. */
int sph_batch_get_field(sph_ctx* ctx, int32_t inst, int32_t field, double* out);

/* Counts, steps taken, simulated time and Courant statistics of a system. */
int sph_batch_info(sph_ctx* ctx, int32_t inst, int64_t* n_real, int64_t* n_wall,
                   int64_t* step, double* time, double* max_courant, double* mean_courant);

/* Free room: real and wall particle slots and instance slots. */
int sph_batch_capacity(sph_ctx* ctx, int64_t* free_real, int64_t* free_wall,
                       int32_t* free_slots);

/* Number of instance slots of a batch and, in `live` (max_instances bytes,
 * may be NULL), 1 for each slot that holds a system. */
int sph_batch_slots(sph_ctx* ctx, int32_t* max_instances, uint8_t* live);

/* ---- status, streams, timing ------------------------------------------- */

/* Last error of this context as text; returns the last status code. */
int sph_status(sph_ctx* ctx, char* msg, size_t len);

/* The CUDA stream (cudaStream_t as void*) the context launches on. */
int sph_get_stream(sph_ctx* ctx, void** stream);

/* Per-stage timing: when enabled, every step records CUDA events around
 * each stage on the context stream.  sph_stage_times returns the summed
 * milliseconds of each stage since the last reset (SPH_STAGE_* order) and
 * the number of steps they cover. */
#define SPH_STAGE_HASH     0   /* cell keys + radix sort + cell ranges     */
#define SPH_STAGE_PERMUTE  1   /* reorder state + half-kick                */
#define SPH_STAGE_PASS_A   2   /* density / divergence / strain rate + EOS */
#define SPH_STAGE_PASS_B   3   /* forces                                   */
#define SPH_STAGE_UPDATE   4   /* leap-frog update + reductions            */
#define SPH_NUM_STAGES     5
int sph_enable_stage_timing(sph_ctx* ctx, int32_t on);
int sph_stage_times(sph_ctx* ctx, double ms[SPH_NUM_STAGES], int64_t* steps);

/* Context options.
 *  SPH_OPT_GRAPHS: 1 (default) replays steady-state steps of sph_advance as a
 *    captured CUDA graph of two steps; 0 launches every kernel eagerly.
 *  SPH_OPT_SMEM_CARVEOUT: percentage of the unified L1/shared storage the
 *    pair passes prefer as shared memory (cudaFuncAttributePreferredShared-
 *    MemoryCarveout; -1 = driver default).  A tuning knob of the autotuner. */
#define SPH_OPT_GRAPHS          1
#define SPH_OPT_SMEM_CARVEOUT   2
/*  SPH_OPT_BLOCK_SIZE: threads per block of the mixed-precision pair passes
 *    (32, 64, 128 (default) or 256).
 *  SPH_OPT_LIST_LEN: neighbour-list entries per lane of those passes: 64,
 *    88 or 120 (default 64 in 2-D, 88 in 3-D).  Each block stages
 *    block/32 x (32 x list + 128) words in shared memory (227 KB at most).
 *    Both are tuning knobs of the autotuner; results do not depend on them. */
#define SPH_OPT_BLOCK_SIZE      3
#define SPH_OPT_LIST_LEN        4
/*  SPH_OPT_PERSISTENT: 1 launches the mixed-precision pair passes as
 *    persistent grids (only the blocks the device holds at once, each
 *    striding over the tiles of targets); 0 (default) one block per tile.
 *    Results do not depend on it. */
#define SPH_OPT_PERSISTENT      5
/*  SPH_OPT_LANES: lanes per target of the FP64 passes A and B: 1 (default),
 *    2, 4, 8, 16 or 32.  With L lanes each target's neighbours are dealt
 *    round-robin, in the walk's order, over L lanes of a warp, and the L
 *    partial sums are added by a fixed butterfly: a small system (a few
 *    thousand particles, where one lane's chain of pair arithmetic sets the
 *    time of a pass) runs on L times as many warps.  The summation order
 *    depends on L and on nothing else, so results differ from L = 1 by
 *    rounding only and are the same on every run and alone or in a batch
 *    with the same L.  It applies to the SPH = 2 form without kernel
 *    correction or artificial heat; the other forms and precisions run one
 *    lane per target. */
#define SPH_OPT_LANES           6
int sph_set_option(sph_ctx* ctx, int32_t option, double value);

/* Number of kernel launches issued by this context since creation. */
int sph_launch_count(sph_ctx* ctx, int64_t* count);

/* Device memory held by the context, in bytes. */
int sph_device_bytes(sph_ctx* ctx, int64_t* bytes);

/* The parameters the context was created (or last set) with. */
int sph_get_params(sph_ctx* ctx, sph_params* out);

/* ---- state snapshots (checkpoint / resume) ------------------------------- *
 * The reference restarts from particle files written by output()
 * (src/Output/output.f90:7-83; readInitialFile, input.f90:22-43), which hold
 * neither the last step's rates nor the leap-frog and Courant state.  A
 * snapshot holds the full state of a context (plain or batch) between steps,
 * so a resumed run continues bit for bit: the live particle slots in their
 * cell order, the last step's rates, the wall data, the instance and
 * material tables, the step counters and the Courant statistics.
 * sph_state_bytes gives the size; sph_state_save writes it into a host
 * buffer; sph_state_load creates a new context on the current device from
 * one (same library build; SPH_E_INVALID otherwise).  The options of
 * sph_set_option are not state: a loaded context starts from their defaults
 * (with SPH_OPT_LANES, set it again to continue with the same bits). */
int sph_state_bytes(sph_ctx* ctx, int64_t* bytes);
int sph_state_save(sph_ctx* ctx, void* buffer, int64_t size);
int sph_state_load(const void* buffer, int64_t size, sph_ctx** out);

/* ---- stand-alone cell-hash sort ----------------------------------------- *
 * Stable LSD radix sort of (key, value) pairs on device memory, the sort
 * that orders particles by cell.  Device pointers; `scratch` must hold
 * sph_sort_scratch_bytes(n, key_bits) bytes; sorted output lands in
 * keys_out / vals_out.  `stream` is a cudaStream_t (NULL = default). */
int64_t sph_sort_scratch_bytes(int64_t n, int32_t key_bits);
int sph_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in,
                   uint32_t* keys_out, uint32_t* vals_out, int64_t n,
                   int32_t key_bits, void* scratch, int64_t scratch_bytes,
                   void* stream);

/* Allocation-free variant of sph_sort_pairs.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc — a host whose
 * device memory is owned by another allocator (a framework's caching pool that
 * holds the whole device, a fixed memory budget), or a latency-critical loop
 * where an allocation, which may synchronise the device, is not allowed.
 * The scratch is one file-scope device array of the library sized for
 * SPH_NOALLOC_MAX_PAIRS pairs (8,651,008 bytes, about 8.65 MB or 8.25 MiB,
 * held on every device that loads the library until the process exits);
 * larger inputs are rejected with SPH_E_TOO_LARGE before any work is queued.
 * The caller still passes device pointers for the keys and values in and
 * out.  The first call on a device looks the array's device address up (with
 * that device current), so make that first call before any stream capture.
 * Later calls outside a capture look it up again, so a device reset
 * (cudaDeviceReset) between calls is picked up; a call under capture reuses
 * the address of the device's last call outside capture.  Every call
 * shares the one array: calls that overlap on the GPU (other streams, other
 * host threads on the same device) race and must be serialised by the
 * caller.  No cudaMalloc, cudaFree or allocating library routine is called. */
#define SPH_NOALLOC_MAX_PAIRS (1 << 20)
int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in,
                           uint32_t* keys_out, uint32_t* vals_out, int64_t n,
                           int32_t key_bits, void* stream);

/* ---- micro-benchmarks used for the roofline denominators ---------------- */

/* Measured FP64 FMA throughput of the current device in GFLOP/s (2 flops
 * per FMA), from a register-resident FMA-chain kernel timed with events. */
int sph_probe_fp64_gflops(double* gflops);

/* Self-check of the float <-> double conversions that the pair passes form on
 * the integer pipes (on this GPU the conversion instructions issue on the
 * FP64 pipe): over n seeded cases of each kind (random bit patterns, doubles
 * in the float range, round-half ties and their neighbours, random floats)
 * the count of results whose bits differ from the conversion instructions'
 * (0 when they agree). */
int sph_check_conversions(int64_t n, uint64_t seed, int64_t* mismatches);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GPU_H */
