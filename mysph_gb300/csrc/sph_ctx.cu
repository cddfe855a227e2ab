// sph_ctx.cu — contexts and the extern "C" entry points of libsphgpu.so.
//
// A context owns one particle system on one GPU: device state in cell order
// (see sph_device.cuh), the static wall hash, scratch of the radix sort and
// one CUDA stream.  Every entry point validates its arguments, returns an
// SPH_* status and never aborts; CUDA errors are turned into SPH_E_CUDA with
// the message kept for sph_status.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sph_gpu.h"
#include "sph_device.cuh"
#include "sph_internal.h"
#include "sph_kernels.cuh"

using sph::Dev;

struct sph_ctx {
    sph_params prm{};
    Dev d{};
    sph::DevMaterial* d_mat = nullptr;
    int64_t capacity = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;     // particle-sized arrays (freed at destroy)
    std::vector<void*> grid_allocs;
    int64_t grid_cells_alloc = -1;
    int64_t device_bytes = 0;
    void* sort_scratch = nullptr;
    int64_t sort_scratch_bytes = 0;
    uint32_t* scan_part = nullptr;
    int64_t scan_part_n = 0;
    double* stage = nullptr;       // staging for uploads / gathers
    int64_t stage_bytes = 0;
    int* d_counts = nullptr;       // neighbour counts in uploaded order
    long long* d_offsets = nullptr;
    int* d_list = nullptr;
    int64_t d_list_cap = 0;
    bool uploaded = false;
    bool hash_valid = false;
    bool rates_valid = false;
    int64_t step = 0;
    double time = 0.0;
    int key_bits = 1;
    int last_status = SPH_OK;
    std::string msg;
    bool timing = false;
    static constexpr int kPool = 64;             // steps of events kept before a flush
    std::vector<cudaEvent_t> ev;                 // kPool * (SPH_NUM_STAGES + 1)
    int ev_used = 0;                             // steps recorded, not yet summed
    double stage_ms[SPH_NUM_STAGES] = {};
    int64_t timed_steps = 0;
    int64_t launches = 0;
};

namespace {

int fail(sph_ctx* c, int st, const std::string& m) {
    if (c) { c->last_status = st; c->msg = m; }
    return st;
}

#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(ctx, SPH_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(sph_ctx* ctx, T** p, int64_t count, std::vector<void*>& list) {
    *p = nullptr;
    if (count <= 0) count = 1;
    size_t bytes = (size_t)count * sizeof(T);
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, SPH_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    list.push_back(*p);
    ctx->device_bytes += (int64_t)bytes;
    return SPH_OK;
}

void free_list(sph_ctx* ctx, std::vector<void*>& list) {
    for (void* p : list) cudaFree(p);
    list.clear();
    (void)ctx;
}

int check_params(const sph_params* p) {
    if (!p) return SPH_E_INVALID;
    if (p->dim != 2 && p->dim != 3) return SPH_E_UNSUPPORTED;
    if (p->skf < 1 || p->skf > 3) return SPH_E_INVALID;
    if (p->pa_sph != 2) return SPH_E_UNSUPPORTED;
    if (p->sle != 0) return SPH_E_UNSUPPORTED;
    if (p->flags & (SPH_F_SUM_DENSITY | SPH_F_AVER_VELOCITY)) return SPH_E_UNSUPPORTED;
    if (p->precision != SPH_PREC_FP64 && p->precision != SPH_PREC_MIXED) return SPH_E_UNSUPPORTED;
    if (p->n_materials < 0 || p->n_materials > SPH_MAX_MATERIALS) return SPH_E_INVALID;
    if (!(p->dt > 0.0)) return SPH_E_INVALID;
    return SPH_OK;
}

// Parameter fields of the device view; the material rows go to `mats`
// (uploaded to the context's device table by upload_materials).
void fill_dev_params(Dev& d, const sph_params& p, sph::DevMaterial* mats) {
    d.dim = p.dim;
    d.precision = p.precision;
    d.d2 = p.dim * p.dim;
    d.skf = p.skf;
    d.pa_sph = p.pa_sph;
    d.sle = p.sle;
    d.flags = p.flags;
    d.scale_k = sph::scale_k_of(p.skf);
    d.dt = p.dt;
    d.gravity = p.gravity;
    d.av_alpha = p.av_alpha; d.av_beta = p.av_beta; d.av_psi = p.av_psi;
    d.av_alpha_solid = p.av_alpha_solid; d.av_beta_solid = p.av_beta_solid;
    d.cour_alpha = p.cour_alpha; d.cour_beta = p.cour_beta;
    d.wall_fs = p.wall_fs; d.wall_r0 = p.wall_r0; d.wall_p1 = p.wall_p1; d.wall_p2 = p.wall_p2;
    d.pen_factor = p.pen_factor; d.pen_n1 = p.pen_n1; d.pen_n2 = p.pen_n2;
    d.contact_delta = p.contact_delta;
    d.as_eps = p.as_eps; d.as_n = p.as_n; d.as_dp = p.as_dp; d.xsph_eps = p.xsph_eps;
    d.n_mat = p.n_materials;
    for (int k = 0; k < p.n_materials; ++k) {
        const sph_material& m = p.materials[k];
        sph::DevMaterial& o = mats[k];
        o.type = m.type; o.eos = m.eos; o.solid = m.solid; o.yield = m.yield;
        o.rho0 = m.rho0; o.c0 = m.c0; o.gamma = m.gamma; o.K = m.K; o.eta = m.eta;
        o.sigma_y = m.sigma_y; o.mg_cs = m.mg_cs; o.mg_s = m.mg_s;
        o.tait_b = m.gamma != 0.0 ? ((m.c0 * m.c0) * m.rho0) / m.gamma : 0.0;
    }
}

// FP32 mirrors of the mixed-precision passes (allocated on first use).
int ensure_mirrors(sph_ctx* ctx) {
    Dev& d = ctx->d;
    const int64_t N = ctx->capacity, D2 = (int64_t)ctx->prm.dim * ctx->prm.dim;
    int st = 0;
    if (!d.pr4) {
        st |= dalloc(ctx, &d.pr4, N, ctx->allocs); st |= dalloc(ctx, &d.vf4, N, ctx->allocs);
        st |= dalloc(ctx, &d.ef4, N, ctx->allocs); st |= dalloc(ctx, &d.pf4, N, ctx->allocs);
        st |= dalloc(ctx, &d.tf, N * D2, ctx->allocs);
    }
    if (d.has_solid && !d.sf) {
        st |= dalloc(ctx, &d.sf, N * D2, ctx->allocs);
        st |= dalloc(ctx, &d.rf4, N, ctx->allocs);
    }
    return st ? SPH_E_NOMEM : SPH_OK;
}

int upload_materials(sph_ctx* ctx, const sph_params& p) {
    sph::DevMaterial mats[SPH_MAX_MATERIALS] = {};
    fill_dev_params(ctx->d, p, mats);
    ctx->d.mat = ctx->d_mat;
    CK(cudaMemcpyAsync(ctx->d_mat, mats, sizeof(mats), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// Stage timing: record event k of the current step on the context stream.
// Events are summed lazily (flush_timing), so timing adds no host sync.
inline void mark(sph_ctx* ctx, int k) {
    if (ctx->timing) cudaEventRecord(ctx->ev[ctx->ev_used * (SPH_NUM_STAGES + 1) + k], ctx->stream);
}

void flush_timing(sph_ctx* ctx) {
    if (!ctx->ev_used) return;
    cudaEventSynchronize(ctx->ev[ctx->ev_used * (SPH_NUM_STAGES + 1) - 1]);
    for (int st = 0; st < ctx->ev_used; ++st)
        for (int k = 0; k < SPH_NUM_STAGES; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev[st * (SPH_NUM_STAGES + 1) + k], ctx->ev[st * (SPH_NUM_STAGES + 1) + k + 1]);
            ctx->stage_ms[k] += ms;
        }
    ctx->timed_steps += ctx->ev_used;
    ctx->ev_used = 0;
}

void swap_buffers(Dev& d) {
    std::swap(d.xm, d.xm2);
    std::swap(d.vr, d.vr2);
    std::swap(d.eh, d.eh2);
    std::swap(d.dsp, d.dsp2);
    std::swap(d.meta, d.meta2);
    std::swap(d.shear, d.shear2);
}

// Cell keys, radix sort, cell starts and the reorder of the real particles
// (with the half kick when `kick`).
int build_hash(sph_ctx* ctx, bool kick) {
    Dev& d = ctx->d;
    cudaStream_t s = ctx->stream;
    if (d.n_real == 0) { ctx->hash_valid = true; return SPH_OK; }
    CK(cudaMemsetAsync(d.ccount, 0, sizeof(int) * ((size_t)d.grid.ncells + 1), s));
    sph::launch_keys(d, d.n_real, d.xm, d.meta, d.keys, d.vals, d.ccount, s);
    cudaError_t e = sph::sort_pairs(d.keys, d.vals, d.keys_s, d.vals_s, d.n_real, ctx->key_bits,
                                    ctx->sort_scratch, s, &ctx->launches);
    if (e != cudaSuccess) return fail(ctx, SPH_E_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
    sph::exclusive_scan_u32((const uint32_t*)d.ccount, (uint32_t*)d.fstart, (int64_t)d.grid.ncells + 1,
                            ctx->scan_part, s, &ctx->launches);
    mark(ctx, 1);
    sph::launch_permute(d, kick, s);
    swap_buffers(d);
    ctx->launches += 3;
    CK(cudaGetLastError());
    ctx->hash_valid = true;
    return SPH_OK;
}

int need(sph_ctx* ctx, bool hash) {
    if (!ctx) return SPH_E_INVALID;
    if (!ctx->uploaded) return fail(ctx, SPH_E_STATE, "no particles uploaded");
    if (hash && !ctx->hash_valid) return fail(ctx, SPH_E_STATE, "call sph_nnps first");
    return SPH_OK;
}

int gather_to_host(sph_ctx* ctx, int field, double* out, int64_t count) {
    if (!out) return SPH_OK;
    sph::launch_gather_field(ctx->d, field, ctx->stage, ctx->stream);
    ++ctx->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, ctx->stage, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int comps_of(const Dev& d, int field) {
    switch (field) {
    case SPH_FIELD_X: case SPH_FIELD_V: case SPH_FIELD_DISP: case SPH_FIELD_DVDT: return d.dim;
    case SPH_FIELD_STRESS: case SPH_FIELD_SHEAR: case SPH_FIELD_DSDT: case SPH_FIELD_STRAIN: return d.d2;
    default: return 1;
    }
}

int check_status_word(sph_ctx* ctx) {
    uint32_t st = 0;
    CK(cudaMemcpyAsync(&st, ctx->d.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st & sph::ST_NONFINITE) return fail(ctx, SPH_E_NONFINITE, "non-finite rho, v, e or x after a step");
    return SPH_OK;
}

int run_passes(sph_ctx* ctx, uint32_t terms, bool assemble, bool strain) {
    Dev& d = ctx->d;
    mark(ctx, 2);
    sph::launch_pass_a(d, strain, ctx->stream);
    mark(ctx, 3);
    sph::launch_pass_b(d, terms, assemble, ctx->stream);
    mark(ctx, 4);
    ctx->launches += 2;
    CK(cudaGetLastError());
    return SPH_OK;
}

int one_step(sph_ctx* ctx) {
    Dev& d = ctx->d;
    const bool first = ctx->step == 0;
    mark(ctx, 0);
    int st = build_hash(ctx, !first);
    if (st) return st;
    st = run_passes(ctx, sph::step_terms(d), true, false);
    if (st) return st;
    int nb = 0;
    sph::launch_update(d, first, ctx->stream, &nb);
    ++ctx->launches;
    if (!first) {
        sph::launch_courant_final(d, nb, ctx->stream);
        ++ctx->launches;
    }
    mark(ctx, 5);
    CK(cudaGetLastError());
    if (ctx->timing && ++ctx->ev_used == sph_ctx::kPool) flush_timing(ctx);
    ctx->step += 1;
    ctx->time += d.dt;
    ctx->hash_valid = false;
    ctx->rates_valid = true;
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }

int sph_params_default(sph_params* p) {
    if (!p) return SPH_E_INVALID;
    std::memset(p, 0, sizeof(*p));
    p->dim = 2;
    p->skf = 1;
    p->pa_sph = 2;
    p->sle = 0;
    p->flags = SPH_F_SUM_DENSITY;  // getValueFromToml.f90:135
    p->precision = SPH_PREC_FP64;
    p->dt = 5e-4;                  // :129 default dble(5e-4)
    p->gravity = -9.81;
    p->av_alpha = 1.0; p->av_beta = 1.0; p->av_psi = (double)0.1f;
    p->av_alpha_solid = 1.0; p->av_beta_solid = 1.0;
    p->cour_alpha = 1.0; p->cour_beta = 1.0;
    p->wall_fs = (double)1e-2f; p->wall_r0 = (double)1.25e-5f; p->wall_p1 = 12; p->wall_p2 = 4;
    p->pen_factor = 1e5; p->pen_n1 = 6; p->pen_n2 = 4;
    p->contact_delta = (double)0.001f;
    p->as_eps = (double)0.2f; p->as_n = 4; p->as_dp = 0.0;
    p->xsph_eps = (double)0.3f;
    p->n_materials = 1;
    p->materials[0].type = 2;
    p->materials[0].eos = SPH_EOS_TAIT;
    p->materials[0].rho0 = 1000.0;
    p->materials[0].gamma = 7.0;
    p->materials[0].eta = (double)1e-3f;
    return SPH_OK;
}

int sph_create(const sph_params* prm, int64_t capacity, sph_ctx** out) {
    if (!out) return SPH_E_INVALID;
    *out = nullptr;
    int st = check_params(prm);
    if (st) return st;
    if (capacity <= 0 || capacity >= ((int64_t)1 << 31)) return SPH_E_INVALID;
    sph_ctx* ctx = new sph_ctx();
    ctx->prm = *prm;
    ctx->capacity = capacity;
    cudaGetDevice(&ctx->device);
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete ctx; return SPH_E_CUDA; }
    Dev& d = ctx->d;
    const int64_t N = capacity;
    const int64_t D2 = (int64_t)prm->dim * prm->dim;
    auto& L = ctx->allocs;
    st = 0;
    st |= dalloc(ctx, &d.xm, N, L); st |= dalloc(ctx, &d.vr, N, L); st |= dalloc(ctx, &d.eh, N, L);
    st |= dalloc(ctx, &d.dsp, N, L); st |= dalloc(ctx, &d.meta, N, L);
    st |= dalloc(ctx, &d.xm2, N, L); st |= dalloc(ctx, &d.vr2, N, L); st |= dalloc(ctx, &d.eh2, N, L);
    st |= dalloc(ctx, &d.dsp2, N, L); st |= dalloc(ctx, &d.meta2, N, L);
    st |= dalloc(ctx, &d.posf, N, L); st |= dalloc(ctx, &d.pa4, N, L); st |= dalloc(ctx, &d.tt, N * D2, L);
    st |= dalloc(ctx, &d.dvr, N, L); st |= dalloc(ctx, &d.dedt, N, L); st |= dalloc(ctx, &d.tds, N, L);
    st |= dalloc(ctx, &d.prev_vr, N, L); st |= dalloc(ctx, &d.prev_e, N, L);
    st |= dalloc(ctx, &d.keys, N, L); st |= dalloc(ctx, &d.vals, N, L);
    st |= dalloc(ctx, &d.keys_s, N, L); st |= dalloc(ctx, &d.vals_s, N, L);
    st |= dalloc(ctx, &d.nneigh, N, L);
    st |= dalloc(ctx, &d.red, 2 * (N / 256 + 2), L);
    st |= dalloc(ctx, &d.courant, 4, L);
    st |= dalloc(ctx, &d.status, 1, L);
    st |= dalloc(ctx, &ctx->d_mat, SPH_MAX_MATERIALS, L);
    st |= dalloc(ctx, &ctx->d_counts, N, L);
    st |= dalloc(ctx, &ctx->d_offsets, N + 1, L);
    ctx->stage_bytes = sizeof(double) * N * std::max<int64_t>(D2, 2 * prm->dim + 2) + 64;
    st |= dalloc(ctx, (char**)&ctx->stage, ctx->stage_bytes, L);
    ctx->sort_scratch_bytes = sph::sort_scratch_bytes(N, 32);
    st |= dalloc(ctx, (char**)&ctx->sort_scratch, ctx->sort_scratch_bytes, L);
    if (st) {
        free_list(ctx, ctx->allocs);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return SPH_E_NOMEM;
    }
    cudaMemsetAsync(d.courant, 0, 4 * sizeof(double), ctx->stream);
    cudaMemsetAsync(d.status, 0, sizeof(uint32_t), ctx->stream);
    if ((prm->precision == SPH_PREC_MIXED && ensure_mirrors(ctx) != SPH_OK) ||
        upload_materials(ctx, *prm) != SPH_OK) {
        free_list(ctx, ctx->allocs);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return SPH_E_CUDA;
    }
    ctx->ev.resize((size_t)sph_ctx::kPool * (SPH_NUM_STAGES + 1));
    for (auto& e2 : ctx->ev) cudaEventCreate(&e2);
    *out = ctx;
    return SPH_OK;
}

int sph_destroy(sph_ctx* ctx) {
    if (!ctx) return SPH_E_INVALID;
    cudaStreamSynchronize(ctx->stream);
    free_list(ctx, ctx->allocs);
    free_list(ctx, ctx->grid_allocs);
    for (auto& e2 : ctx->ev)
        if (e2) cudaEventDestroy(e2);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SPH_OK;
}

int sph_set_params(sph_ctx* ctx, const sph_params* prm) {
    if (!ctx) return SPH_E_INVALID;
    int st = check_params(prm);
    if (st) return fail(ctx, st, "unsupported parameters");
    if (prm->dim != ctx->prm.dim) return fail(ctx, SPH_E_INVALID, "dim cannot change");
    const bool to_mixed = prm->precision == SPH_PREC_MIXED && ctx->prm.precision != SPH_PREC_MIXED;
    ctx->prm = *prm;
    if (prm->precision == SPH_PREC_MIXED && ensure_mirrors(ctx)) return fail(ctx, SPH_E_NOMEM, "FP32 mirrors");
    st = upload_materials(ctx, *prm);  // parameter fields only; pointers and grid stay
    if (st) return st;
    if (to_mixed && ctx->uploaded) {
        // wall mirrors are written once; real particles' at the next reorder
        sph::launch_wall_init(ctx->d, ctx->stream);
        ctx->hash_valid = false;
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return SPH_OK;
}

int sph_upload(sph_ctx* ctx, int64_t n_real, int64_t n_wall, const double* x, const double* v,
               const double* mass, const double* rho, const double* p, const double* e, const double* c,
               const double* h, const int32_t* type, const int32_t* state, const int32_t* boundary,
               const double* shear) {
    if (!ctx) return SPH_E_INVALID;
    if (n_real < 0 || n_wall < 0 || n_real + n_wall <= 0 || n_real + n_wall > ctx->capacity)
        return fail(ctx, SPH_E_INVALID, "particle count out of range");
    if (!x || !v || !mass || !rho || !p || !e || !c || !h || !type)
        return fail(ctx, SPH_E_INVALID, "null input array");
    Dev& d = ctx->d;
    const int dim = ctx->prm.dim, D2 = dim * dim;
    const int64_t N = n_real + n_wall;
    // host-side scan: bounding box, smoothing lengths, solids, finiteness
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, hmax = 0.0, hmin = 1e300;
    bool solid = false;
    for (int a = 0; a < dim; ++a) { lo[a] = 1e300; hi[a] = -1e300; }
    for (int64_t i = 0; i < N; ++i) {
        for (int a = 0; a < dim; ++a) {
            double xv = x[i * dim + a];
            if (!std::isfinite(xv)) return fail(ctx, SPH_E_INVALID, "non-finite position");
            lo[a] = std::min(lo[a], xv);
            hi[a] = std::max(hi[a], xv);
        }
        if (!(h[i] > 0.0) || !std::isfinite(h[i])) return fail(ctx, SPH_E_INVALID, "smoothing length must be > 0");
        if (!(rho[i] > 0.0)) return fail(ctx, SPH_E_INVALID, "density must be > 0");
        hmax = std::max(hmax, h[i]);
        hmin = std::min(hmin, h[i]);
        if (std::abs(type[i]) > 100) solid = true;
    }
    const sph_params& P = ctx->prm;
    const double reach_max = hmax * sph::scale_k_of(P.skf);
    double cs = P.cell_size > 0.0 ? P.cell_size : reach_max * (1.0 + 1e-9);
    if (cs < reach_max) return fail(ctx, SPH_E_INVALID, "cell_size below scale_k * max(h)");
    bool user_domain = true;
    for (int a = 0; a < dim; ++a)
        if (!(P.domain_lo[a] < P.domain_hi[a])) user_domain = false;
    double margin = P.grid_margin > 0.0 ? P.grid_margin : 2.0 * cs;
    sph::Grid g{};
    int64_t ncells = 1;
    for (;;) {
        ncells = 1;
        for (int a = 0; a < 3; ++a) {
            if (a >= dim) { g.lo[a] = 0.0; g.nc[a] = 1; continue; }
            double l = user_domain ? P.domain_lo[a] : lo[a] - margin;
            double u = user_domain ? P.domain_hi[a] : hi[a] + margin;
            g.lo[a] = l;
            int64_t nc = (int64_t)std::ceil((u - l) / cs);
            nc = std::max<int64_t>(nc, 1);
            g.nc[a] = (int)std::min<int64_t>(nc, 1 << 24);
            ncells *= g.nc[a];
        }
        if (ncells <= (int64_t)16 * 1024 * 1024 - 2) break;
        cs *= 1.25;  // very sparse domains: coarser cells (still exact)
    }
    g.cs = cs;
    g.inv_cs = 1.0 / cs;
    g.ncells = (int)ncells;
    double ext = 0.0;
    for (int a = 0; a < dim; ++a) ext = std::max(ext, g.nc[a] * cs);
    // FP32 filter guard on r^2 (relative): positions rounded to FP32 relative
    // to the grid origin err by ext*2^-24 each, so |dx| errs by sqrt(dim)*ext*2^-23
    const double reach_min = hmin * sph::scale_k_of(P.skf);
    const double delta = std::sqrt((double)dim) * ext * std::ldexp(1.0, -23);
    double guard = 2.0 * (2.0 * delta / reach_min + (delta / reach_min) * (delta / reach_min) + std::ldexp(1.0, -19));
    if (guard > 0.5) guard = 1e30;  // filter useless: always take the exact test
    g.guard = (float)guard;
    d.grid = g;
    d.n_real = (int)n_real;
    d.n_wall = (int)n_wall;
    d.n = (int)N;
    ctx->key_bits = 1;
    while (((int64_t)1 << ctx->key_bits) <= ncells) ++ctx->key_bits;
    // grid arrays
    if (ncells + 1 > ctx->grid_cells_alloc) {
        free_list(ctx, ctx->grid_allocs);
        int st = 0;
        st |= dalloc(ctx, &d.fstart, ncells + 2, ctx->grid_allocs);
        st |= dalloc(ctx, &d.wstart, ncells + 2, ctx->grid_allocs);
        st |= dalloc(ctx, &d.ccount, ncells + 2, ctx->grid_allocs);
        int64_t np = sph::scan_partials(std::max<int64_t>(ncells + 2, ctx->capacity * 256 / 4096 + 256));
        st |= dalloc(ctx, &ctx->scan_part, np, ctx->grid_allocs);
        if (st) return fail(ctx, SPH_E_NOMEM, "grid allocation failed");
        ctx->grid_cells_alloc = ncells + 1;
    }
    // solid arrays
    if (solid && !d.has_solid) {
        int st = 0;
        st |= dalloc(ctx, &d.shear, ctx->capacity * D2, ctx->allocs);
        st |= dalloc(ctx, &d.shear2, ctx->capacity * D2, ctx->allocs);
        st |= dalloc(ctx, &d.sig, ctx->capacity * D2, ctx->allocs);
        st |= dalloc(ctx, &d.dsdt, ctx->capacity * D2, ctx->allocs);
        st |= dalloc(ctx, &d.shear_prev, ctx->capacity * D2, ctx->allocs);
        st |= dalloc(ctx, &d.ras, ctx->capacity, ctx->allocs);
        if (st) return fail(ctx, SPH_E_NOMEM, "solid arrays");
        d.has_solid = 1;
    }
    if (ctx->prm.precision == SPH_PREC_MIXED && ensure_mirrors(ctx))
        return fail(ctx, SPH_E_NOMEM, "FP32 mirrors");
    if (!d.strain) {
        if (dalloc(ctx, &d.strain, ctx->capacity * D2, ctx->allocs)) return fail(ctx, SPH_E_NOMEM, "strain");
    }
    // host -> device staging (x, v, m, rho, p, e, c, h, shear | type, state, bnd)
    std::vector<void*> tmp;
    double *dx_ = nullptr, *dv_ = nullptr, *dsc = nullptr, *dsh = nullptr;
    int *dt_ = nullptr;
    uint32_t* word = nullptr;
    int st = 0;
    st |= dalloc(ctx, &dx_, N * dim, tmp);
    st |= dalloc(ctx, &dv_, N * dim, tmp);
    st |= dalloc(ctx, &dsc, N * 6, tmp);
    st |= dalloc(ctx, &dt_, N * 3, tmp);
    if (shear && d.has_solid) st |= dalloc(ctx, &dsh, N * D2, tmp);
    st |= dalloc(ctx, &word, N * 2, tmp);
    if (st) { free_list(ctx, tmp); return fail(ctx, SPH_E_NOMEM, "upload staging"); }
    cudaStream_t s = ctx->stream;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
    };
    cudaError_t ce = cudaSuccess;
    ce = up(dx_, x, sizeof(double) * N * dim); if (ce) goto cuda_fail;
    ce = up(dv_, v, sizeof(double) * N * dim); if (ce) goto cuda_fail;
    ce = up(dsc + 0 * N, mass, sizeof(double) * N); if (ce) goto cuda_fail;
    ce = up(dsc + 1 * N, rho, sizeof(double) * N); if (ce) goto cuda_fail;
    ce = up(dsc + 2 * N, p, sizeof(double) * N); if (ce) goto cuda_fail;
    ce = up(dsc + 3 * N, e, sizeof(double) * N); if (ce) goto cuda_fail;
    ce = up(dsc + 4 * N, c, sizeof(double) * N); if (ce) goto cuda_fail;
    ce = up(dsc + 5 * N, h, sizeof(double) * N); if (ce) goto cuda_fail;
    ce = up(dt_, type, sizeof(int) * N); if (ce) goto cuda_fail;
    if (state) { ce = up(dt_ + N, state, sizeof(int) * N); if (ce) goto cuda_fail; }
    if (boundary) { ce = up(dt_ + 2 * N, boundary, sizeof(int) * N); if (ce) goto cuda_fail; }
    if (dsh) { ce = up(dsh, shear, sizeof(double) * N * D2); if (ce) goto cuda_fail; }
    {
        uint32_t* worder = word;            // wall order (n_wall)
        uint32_t* wkeys = word + N;
        // 1) pack with identity wall order
        ce = cudaMemsetAsync(d.status, 0, sizeof(uint32_t), s); if (ce) goto cuda_fail;
        std::vector<uint32_t> iota(std::max<int64_t>(n_wall, 1));
        for (int64_t k = 0; k < n_wall; ++k) iota[k] = (uint32_t)k;
        if (n_wall > 0) { ce = up(worder, iota.data(), sizeof(uint32_t) * n_wall); if (ce) goto cuda_fail; }
        ce = cudaStreamSynchronize(s); if (ce) goto cuda_fail;
        sph::launch_pack_upload(d, (int)n_real, dx_, dv_, dsc, dsc + N, dsc + 2 * N, dsc + 3 * N, dsc + 4 * N,
                                dsc + 5 * N, dt_, state ? dt_ + N : nullptr, boundary ? dt_ + 2 * N : nullptr,
                                dsh, worder, s);
        ++ctx->launches;
        // 2) wall keys -> sort -> wall order, wall cell starts
        ce = cudaMemsetAsync(d.ccount, 0, sizeof(int) * ((size_t)ncells + 1), s); if (ce) goto cuda_fail;
        if (n_wall > 0) {
            sph::launch_keys(d, (int)n_wall, d.xm + n_real, d.meta + n_real, d.keys, d.vals, d.ccount, s);
            ce = sph::sort_pairs(d.keys, d.vals, wkeys, worder, n_wall, ctx->key_bits, ctx->sort_scratch, s,
                                 &ctx->launches);
            if (ce) goto cuda_fail;
            ++ctx->launches;
        }
        sph::exclusive_scan_u32((const uint32_t*)d.ccount, (uint32_t*)d.wstart, ncells + 1, ctx->scan_part, s,
                                &ctx->launches);
        // 3) pack again with the walls in cell order
        sph::launch_pack_upload(d, (int)n_real, dx_, dv_, dsc, dsc + N, dsc + 2 * N, dsc + 3 * N, dsc + 4 * N,
                                dsc + 5 * N, dt_, state ? dt_ + N : nullptr, boundary ? dt_ + 2 * N : nullptr,
                                dsh, worder, s);
        sph::launch_wall_init(d, s);
        ctx->launches += 2;
        ce = cudaMemsetAsync(d.courant, 0, 4 * sizeof(double), s); if (ce) goto cuda_fail;
        ce = cudaGetLastError(); if (ce) goto cuda_fail;
        ce = cudaStreamSynchronize(s); if (ce) goto cuda_fail;
    }
    free_list(ctx, tmp);
    ctx->uploaded = true;
    ctx->hash_valid = false;
    ctx->rates_valid = false;
    ctx->step = 0;
    ctx->time = 0.0;
    return SPH_OK;
cuda_fail:
    cudaStreamSynchronize(s);
    free_list(ctx, tmp);
    return fail(ctx, SPH_E_CUDA, std::string("upload: ") + cudaGetErrorString(ce));
}

int sph_download(sph_ctx* ctx, double* x, double* v, double* rho, double* p, double* e, double* c,
                 double* shear) {
    int st = need(ctx, false);
    if (st) return st;
    const int64_t N = ctx->d.n, dim = ctx->d.dim;
    if ((st = gather_to_host(ctx, SPH_FIELD_X, x, N * dim))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_V, v, N * dim))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_RHO, rho, N))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_P, p, N))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_E, e, N))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_C, c, N))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_SHEAR, shear, N * dim * dim))) return st;
    return SPH_OK;
}

int sph_get_field(sph_ctx* ctx, int32_t field, double* out) {
    int st = need(ctx, false);
    if (st) return st;
    if (!out || field < SPH_FIELD_X || field > SPH_FIELD_STRAIN) return fail(ctx, SPH_E_INVALID, "bad field");
    return gather_to_host(ctx, field, out, (int64_t)ctx->d.n * comps_of(ctx->d, field));
}

int sph_set_field(sph_ctx* ctx, int32_t field, const double* in) {
    int st = need(ctx, false);
    if (st) return st;
    if (!in) return fail(ctx, SPH_E_INVALID, "null input");
    const int64_t count = (int64_t)ctx->d.n * comps_of(ctx->d, field);
    CK(cudaMemcpyAsync(ctx->stage, in, sizeof(double) * count, cudaMemcpyHostToDevice, ctx->stream));
    sph::launch_set_field(ctx->d, field, ctx->stage, ctx->d.n, ctx->stream);
    ++ctx->launches;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    if (field == SPH_FIELD_X || field == SPH_FIELD_H) ctx->hash_valid = false;
    return SPH_OK;
}

int sph_info(sph_ctx* ctx, int64_t* n_real, int64_t* n_wall, int64_t* step, double* time) {
    if (!ctx) return SPH_E_INVALID;
    if (n_real) *n_real = ctx->d.n_real;
    if (n_wall) *n_wall = ctx->d.n_wall;
    if (step) *step = ctx->step;
    if (time) *time = ctx->time;
    return SPH_OK;
}

int sph_nnps(sph_ctx* ctx) {
    int st = need(ctx, false);
    if (st) return st;
    st = build_hash(ctx, false);
    if (st) return st;
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_neighbor_counts(sph_ctx* ctx, int32_t* counts, int64_t* total) {
    int st = need(ctx, true);
    if (st) return st;
    const int64_t nr = ctx->d.n_real;
    sph::launch_count_neighbors(ctx->d, ctx->d_counts, ctx->stream);
    ++ctx->launches;
    CK(cudaGetLastError());
    std::vector<int32_t> h(std::max<int64_t>(nr, 1));
    CK(cudaMemcpyAsync(h.data(), ctx->d_counts, sizeof(int32_t) * nr, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int64_t t = 0;
    for (int64_t i = 0; i < nr; ++i) t += h[i];
    if (counts) std::memcpy(counts, h.data(), sizeof(int32_t) * nr);
    if (total) *total = t;
    return SPH_OK;
}

int sph_export_neighbors(sph_ctx* ctx, int64_t* offsets, int32_t* list, int64_t capacity) {
    int st = need(ctx, true);
    if (st) return st;
    if (!offsets || (!list && capacity > 0)) return fail(ctx, SPH_E_INVALID, "null output");
    const int64_t nr = ctx->d.n_real;
    std::vector<int32_t> cnt(std::max<int64_t>(nr, 1));
    int64_t total = 0;
    if ((st = sph_neighbor_counts(ctx, cnt.data(), &total))) return st;
    offsets[0] = 0;
    for (int64_t i = 0; i < nr; ++i) offsets[i + 1] = offsets[i] + cnt[i];
    if (total > capacity) return fail(ctx, SPH_E_OVERFLOW, "neighbour list capacity too small");
    if (total > ctx->d_list_cap) {
        if (ctx->d_list) { cudaFree(ctx->d_list); ctx->d_list = nullptr; }
        if (cudaMalloc((void**)&ctx->d_list, sizeof(int) * std::max<int64_t>(total, 1)) != cudaSuccess) {
            cudaGetLastError();
            ctx->d_list_cap = 0;
            return fail(ctx, SPH_E_NOMEM, "neighbour export buffer");
        }
        ctx->d_list_cap = total;
    }
    static_assert(sizeof(long long) == sizeof(int64_t), "int64");
    CK(cudaMemcpyAsync(ctx->d_offsets, offsets, sizeof(int64_t) * (nr + 1), cudaMemcpyHostToDevice, ctx->stream));
    sph::launch_export_neighbors(ctx->d, ctx->d_offsets, ctx->d_list, ctx->stream);
    ++ctx->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(list, ctx->d_list, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

static int module_call(sph_ctx* ctx, uint32_t terms, bool assemble) {
    int st = need(ctx, true);
    if (st) return st;
    return run_passes(ctx, terms, assemble, true);
}

int sph_density(sph_ctx* ctx, double* drhodt) {
    int st = module_call(ctx, 0, false);
    if (st) return st;
    return gather_to_host(ctx, SPH_FIELD_DRHODT, drhodt, ctx->d.n_real);
}

int sph_divergence(sph_ctx* ctx, double* div_x, double* div_v) {
    int st = module_call(ctx, 0, false);
    if (st) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_DIVX, div_x, ctx->d.n_real))) return st;
    return gather_to_host(ctx, SPH_FIELD_DIVV, div_v, ctx->d.n_real);
}

int sph_internal_force(sph_ctx* ctx, double* dvdt, double* dedt, double* dsdt) {
    int st = module_call(ctx, SPH_TERM_INTERNAL, false);
    if (st) return st;
    const int64_t nr = ctx->d.n_real;
    if ((st = gather_to_host(ctx, SPH_FIELD_DVDT, dvdt, nr * ctx->d.dim))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_DEDT, dedt, nr))) return st;
    return gather_to_host(ctx, SPH_FIELD_DSDT, dsdt, nr * ctx->d.d2);
}

int sph_external_force(sph_ctx* ctx, double* dvdt) {
    int st = module_call(ctx, SPH_TERM_EXTERNAL, false);
    if (st) return st;
    return gather_to_host(ctx, SPH_FIELD_DVDT, dvdt, (int64_t)ctx->d.n_real * ctx->d.dim);
}

int sph_arti_visc(sph_ctx* ctx, double* dvdt, double* dedt) {
    int st = module_call(ctx, SPH_TERM_ARTI_VISC, false);
    if (st) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_DVDT, dvdt, (int64_t)ctx->d.n_real * ctx->d.dim))) return st;
    return gather_to_host(ctx, SPH_FIELD_DEDT, dedt, ctx->d.n_real);
}

int sph_arti_stress(sph_ctx* ctx, double* dvdt) {
    if (ctx && ctx->d.dim != 2) return fail(ctx, SPH_E_UNSUPPORTED, "artificial stress is 2-D only");
    int st = module_call(ctx, SPH_TERM_ARTI_STRESS, false);
    if (st) return st;
    return gather_to_host(ctx, SPH_FIELD_DVDT, dvdt, (int64_t)ctx->d.n_real * ctx->d.dim);
}

int sph_rates(sph_ctx* ctx, double* dvdt, double* drhodt, double* dedt) {
    int st = need(ctx, true);
    if (st) return st;
    if ((st = run_passes(ctx, sph::step_terms(ctx->d), true, true))) return st;
    const int64_t nr = ctx->d.n_real;
    if ((st = gather_to_host(ctx, SPH_FIELD_DVDT, dvdt, nr * ctx->d.dim))) return st;
    if ((st = gather_to_host(ctx, SPH_FIELD_DRHODT, drhodt, nr))) return st;
    return gather_to_host(ctx, SPH_FIELD_DEDT, dedt, nr);
}

int sph_single_step(sph_ctx* ctx) {
    int st = need(ctx, false);
    if (st) return st;
    st = one_step(ctx);
    if (st) return st;
    return check_status_word(ctx);
}

int sph_advance(sph_ctx* ctx, int64_t nsteps, double* max_courant, double* mean_courant) {
    int st = need(ctx, false);
    if (st) return st;
    if (nsteps < 0) return fail(ctx, SPH_E_INVALID, "nsteps < 0");
    for (int64_t k = 0; k < nsteps; ++k)
        if ((st = one_step(ctx))) return st;
    if ((st = check_status_word(ctx))) return st;
    if (max_courant || mean_courant) {
        double cr[4];
        CK(cudaMemcpyAsync(cr, ctx->d.courant, sizeof(cr), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (max_courant) *max_courant = cr[0];
        if (mean_courant) *mean_courant = cr[1];
    }
    return SPH_OK;
}

int sph_step_host(sph_ctx* ctx, int64_t nsteps, double* x, double* v, double* rho, double* e,
                  double* shear) {
    int st = need(ctx, false);
    if (st) return st;
    if (nsteps < 0 || !x || !v || !rho || !e) return fail(ctx, SPH_E_INVALID, "null host array");
    Dev& d = ctx->d;
    const int64_t nr = d.n_real, dim = d.dim;
    cudaStream_t s = ctx->stream;
    double* X = ctx->stage;
    double* V = X + nr * dim;
    double* R = V + nr * dim;
    double* E = R + nr;
    CK(cudaMemcpyAsync(X, x, sizeof(double) * nr * dim, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(V, v, sizeof(double) * nr * dim, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(R, rho, sizeof(double) * nr, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(E, e, sizeof(double) * nr, cudaMemcpyHostToDevice, s));
    sph::launch_host_state(d, true, ctx->stage, s);
    ++ctx->launches;
    if (shear && d.has_solid) {
        CK(cudaStreamSynchronize(s));
        CK(cudaMemcpyAsync(ctx->stage, shear, sizeof(double) * nr * d.d2, cudaMemcpyHostToDevice, s));
        sph::launch_set_field(d, SPH_FIELD_SHEAR, ctx->stage, (int)nr, s);
        ++ctx->launches;
    }
    CK(cudaGetLastError());
    ctx->hash_valid = false;
    for (int64_t k = 0; k < nsteps; ++k)
        if ((st = one_step(ctx))) return st;
    sph::launch_host_state(d, false, ctx->stage, s);
    ++ctx->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(x, X, sizeof(double) * nr * dim, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(v, V, sizeof(double) * nr * dim, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(rho, R, sizeof(double) * nr, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(e, E, sizeof(double) * nr, cudaMemcpyDeviceToHost, s));
    if (shear && d.has_solid) {
        if ((st = gather_to_host(ctx, SPH_FIELD_SHEAR, shear, nr * d.d2))) return st;
    }
    CK(cudaStreamSynchronize(s));
    return check_status_word(ctx);
}

int sph_statistics(sph_ctx* ctx, double out[6]) {
    if (!out) return fail(ctx, SPH_E_INVALID, "null output");
    int st = need(ctx, false);
    if (st) return st;
    if (!ctx->hash_valid && (st = build_hash(ctx, false))) return st;
    const int64_t nr = ctx->d.n_real;
    std::vector<int32_t> cnt(std::max<int64_t>(nr, 1));
    int64_t total = 0;
    if ((st = sph_neighbor_counts(ctx, cnt.data(), &total))) return st;
    int mx = 0, mn = 0x7fffffff;
    int64_t imx = -1, imn = -1, zero = 0;
    for (int64_t i = 0; i < nr; ++i) {
        if (cnt[i] > mx) { mx = cnt[i]; imx = i; }
        if (cnt[i] < mn) { mn = cnt[i]; imn = i; }
        if (cnt[i] == 0) ++zero;
    }
    out[0] = mx; out[1] = mn; out[2] = nr ? (double)total / nr : 0.0; out[3] = (double)zero;
    out[4] = (double)(imx + 1); out[5] = (double)(imn + 1);
    return SPH_OK;
}

int sph_status(sph_ctx* ctx, char* msg, size_t len) {
    if (!ctx) return SPH_E_INVALID;
    if (msg && len) {
        std::snprintf(msg, len, "%s", ctx->msg.c_str());
    }
    return ctx->last_status;
}

int sph_get_stream(sph_ctx* ctx, void** stream) {
    if (!ctx || !stream) return SPH_E_INVALID;
    *stream = (void*)ctx->stream;
    return SPH_OK;
}

int sph_enable_stage_timing(sph_ctx* ctx, int32_t on) {
    if (!ctx) return SPH_E_INVALID;
    cudaStreamSynchronize(ctx->stream);
    ctx->ev_used = 0;
    ctx->timing = on != 0;
    for (int k = 0; k < SPH_NUM_STAGES; ++k) ctx->stage_ms[k] = 0.0;
    ctx->timed_steps = 0;
    return SPH_OK;
}

int sph_stage_times(sph_ctx* ctx, double ms[SPH_NUM_STAGES], int64_t* steps) {
    if (!ctx || !ms) return SPH_E_INVALID;
    flush_timing(ctx);
    for (int k = 0; k < SPH_NUM_STAGES; ++k) ms[k] = ctx->stage_ms[k];
    if (steps) *steps = ctx->timed_steps;
    return SPH_OK;
}

int sph_launch_count(sph_ctx* ctx, int64_t* count) {
    if (!ctx || !count) return SPH_E_INVALID;
    *count = ctx->launches;
    return SPH_OK;
}

int sph_device_bytes(sph_ctx* ctx, int64_t* bytes) {
    if (!ctx || !bytes) return SPH_E_INVALID;
    *bytes = ctx->device_bytes;
    return SPH_OK;
}

int sph_probe_fp64_gflops(double* gflops) {
    if (!gflops) return SPH_E_INVALID;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* sink = nullptr;
    if (cudaMalloc((void**)&sink, sizeof(double)) != cudaSuccess) { cudaGetLastError(); return SPH_E_NOMEM; }
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, iters = 4096;
    sph::launch_fp64_probe(sink, iters, blocks, s);  // warm-up
    cudaEventRecord(a, s);
    sph::launch_fp64_probe(sink, iters, blocks, s);
    cudaEventRecord(b, s);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(s);
    cudaFree(sink);
    if (e != cudaSuccess || ms <= 0.f) return SPH_E_CUDA;
    const double flops = 2.0 * 8.0 * (double)iters * 256.0 * blocks;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return SPH_OK;
}

}  // extern "C"
