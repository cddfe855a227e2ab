// sph_kernels.cuh — launch wrappers of the step kernels (sph_kernels.cu),
// called by the context code (sph_ctx.cu).
#pragma once

#include "sph_device.cuh"

namespace sph {

// Effective force terms of a step, from the flags (singleStep.f90:114-130).
uint32_t step_terms(const Dev& d);

// Cell keys of n particles; mark_outside sets bit 31 of the values of those
// outside their grid (the real-particle hash, read by launch_permute).
void launch_keys(const Dev& d, int n, const double4* xm, const int4* meta, const int* pinst,
                 uint32_t* keys, uint32_t* vals, int* counts, cudaStream_t s, bool mark_outside);
void launch_permute(const Dev& d, bool kick, cudaStream_t s);
// Tiled (mixed) passes: dynamic shared memory of a block with `tpb` threads
// and lists of k entries; the largest dynamic shared memory those kernels
// may use (cudaFuncAttributeMaxDynamicSharedMemorySize); the default list
// length.
size_t tiled_smem_bytes(int tpb, int k);
int set_tiled_smem_limit(size_t bytes);
int default_tile_k(int dim);
// Generated blocks into the staging columns of an upload (see sph_block).
void launch_generate_blocks(const sph_block* blocks, const int64_t* start, int nb, int dim, int64_t N,
                            int64_t n_r, double* x, double* v, double* sc, int* t3, uint32_t* wall_order,
                            cudaStream_t s);
// kernel gradient correction factors of every real particle (pass K)
void launch_kernel_correction(const Dev& d, cudaStream_t s);
// summation density (pass S) and its write-back: two launches
void launch_density(const Dev& d, cudaStream_t s);
// fixedBoundary on a host-order rate array (may be null) and on dvr
void launch_boundary(const Dev& d, double* dv, cudaStream_t s);
// courant_num elementwise
void launch_courant_num(int n, double dt, double ca, double cb, const double* h, const double* dv,
                        const double* c, double* xi, cudaStream_t s);
// SPH = 3: the Riemann continuity rate into dvr.w (before pass A)
void launch_riemann_density(const Dev& d, cudaStream_t s);
void launch_pass_a(const Dev& d, bool want_strain, cudaStream_t s);
void launch_pass_b(const Dev& d, uint32_t terms, bool assemble, cudaStream_t s);
// leap-frog update of every real particle, then per instance the Courant
// statistics and the step counter (two launches)
void launch_update(const Dev& d, cudaStream_t s);
void launch_count_neighbors(const Dev& d, int* counts, cudaStream_t s);
void launch_export_neighbors(const Dev& d, const long long* offsets, int* list, cudaStream_t s);
void launch_wall_init(const Dev& d, int first, int count, cudaStream_t s);
void launch_pack_upload(const Dev& d, int n_r, int n_w, int real_dst, int wall_dst, int inst_id,
                        const double* x, const double* v, const double* m, const double* rho,
                        const double* p, const double* e, const double* c, const double* h,
                        const int* type, const int* state, const int* bnd, const double* shear,
                        const uint32_t* wall_order, cudaStream_t s);
// inst_filter < 0: every instance
void launch_gather_field(const Dev& d, int field, double* out, int inst_filter, cudaStream_t s);
// `limit`: the input covers uploaded indices [0, limit); others are left alone
void launch_set_field(const Dev& d, int field, const double* in, int limit, int inst_filter,
                      cudaStream_t s);
// The reference kernel constants of instance `inst` from the h of its real
// particle `first` (first < 0: none).
void launch_kref(const Dev& d, int inst, int first, cudaStream_t s);
// x, v, rho, e of the real particles between the state and `stage` (in upload
// order): mode 0 state -> stage, 1 stage -> state, 2 the positions alone,
// 3 v, rho and e after 2 (2 and 3 only before a step, whose reorder forms
// the values derived from them).
void launch_host_state(const Dev& d, int mode, double* stage, cudaStream_t s);
// energy sums (kinetic, internal, gravitational) into out[3]; part holds
// 3 doubles per block of 256 real particles; returns the launches issued
int launch_energy(const Dev& d, int inst, double* part, double* out, cudaStream_t s);
// carveout in percent (-1: default) for the pair-pass kernels
void set_pass_carveout(int percent);
void launch_add_offset(int* a, int64_t n, int off, cudaStream_t s);
void launch_fp64_probe(double* sink, int iters, int blocks, cudaStream_t s);
void launch_conversion_check(int64_t n, uint64_t seed, unsigned long long* bad, cudaStream_t s);

}  // namespace sph
