// sph_ctx.cu — contexts and the extern "C" entry points of libsphgpu.so.
//
// A context owns particle systems ("instances") on one GPU: device state in
// cell order (see sph_device.cuh), the static wall hash, scratch of the radix
// sort and one CUDA stream.  A plain context (sph_create + sph_upload) holds
// one instance; a batch context (sph_batch_create + sph_batch_add) holds many
// independent ones that advance together, one launch per stage, each with its
// own grid, material rows and time step.  Every entry point validates its
// arguments, returns an SPH_* status and never aborts; CUDA errors become
// SPH_E_CUDA with the message kept for sph_status.
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

namespace {

// Host record of one instance.
struct HostInst {
    sph::Inst I{};          // mirrored in the device table
    sph_params prm{};
    int64_t n_real = 0, n_wall = 0;
    int64_t wall_first = 0; // slot of its first wall
    bool used = false;      // slot taken (active or removed-but-not-compacted)
};

}  // namespace

struct sph_ctx {
    sph_params prm{};
    Dev d{};
    bool batch = false;
    int max_inst = 1;
    int64_t capacity = 0;       // slots in the particle arrays
    int64_t real_cap = 0;       // batch: slots reserved for real particles
    int64_t wall_end = 0;       // next free wall slot
    int64_t cell_cap = 0;       // cells allocated (cell arrays hold cell_cap + 2)
    int64_t pending_remove = 0; // real particles of removed instances still in [0, n_real)
    std::vector<HostInst> insts;
    sph::DevMaterial* d_mat = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;  // particle-sized arrays (freed at destroy)
    std::vector<void*> grid_allocs;
    int64_t device_bytes = 0;
    void* sort_scratch = nullptr;
    int64_t sort_scratch_bytes = 0;
    uint32_t* scan_part = nullptr;
    double* stage = nullptr;    // staging for uploads / gathers
    int64_t stage_bytes = 0;
    int* d_counts = nullptr;    // neighbour counts in uploaded order
    long long* d_offsets = nullptr;
    int* d_list = nullptr;
    int64_t d_list_cap = 0;
    bool uploaded = false;
    bool hash_valid = false;
    bool density_done = false;  // sum_density ran since the last neighbour search
    bool kgc_done = false;      // kernel-correction factors of this search are current
    int64_t step = 0;           // steps of this context (instance 0 of a plain context)
    double time = 0.0;
    int key_bits = 1;
    int last_status = SPH_OK;
    std::string msg;
    bool timing = false;
    static constexpr int kPool = 64;  // steps of events kept before a flush
    std::vector<cudaEvent_t> ev;      // kPool * (SPH_NUM_STAGES + 1)
    int ev_used = 0;
    double stage_ms[SPH_NUM_STAGES] = {};
    int64_t timed_steps = 0;
    int64_t launches = 0;
    // CUDA graph of two steady-state steps (sph_advance)
    bool use_graphs = true;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_launches = 0;    // kernels in one replay
    int graph_key_bits = 0, graph_n_real = -1, graph_cells = -1;
    const void* graph_xm = nullptr;   // buffer parity the graph was captured with
    const void* graph_dvr = nullptr;
    // sph_step_host: v, rho and e are copied in on a second stream while the
    // cell keys of the uploaded positions are sorted; build_hash writes them
    // into the state before the reorder
    cudaStream_t in_stream = nullptr;
    cudaEvent_t ev_x = nullptr, ev_in = nullptr;
    bool rest_pending = false;
    // build_hash: the scan of the cell counts runs on aux_stream beside the sort
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_keys = nullptr, ev_scan = nullptr;
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

void free_list(std::vector<void*>& list) {
    for (void* p : list) cudaFree(p);
    list.clear();
}

int check_params(const sph_params* p) {
    if (!p) return SPH_E_INVALID;
    if (p->dim != 2 && p->dim != 3) return SPH_E_UNSUPPORTED;
    if (p->skf < 1 || p->skf > 3) return SPH_E_INVALID;
    if (p->pa_sph < 1 || p->pa_sph > 3) return SPH_E_UNSUPPORTED;
    // SPH = 1 and 3 run in FP64, without kernel correction
    if (p->pa_sph != 2 && (p->precision != SPH_PREC_FP64 || (p->flags & SPH_F_KERNEL_CORRECTION)))
        return SPH_E_UNSUPPORTED;
    if (p->sle < 0 || p->sle > 2) return SPH_E_UNSUPPORTED;
    if (p->precision != SPH_PREC_FP64 && p->precision != SPH_PREC_MIXED && p->precision != SPH_PREC_DF64)
        return SPH_E_UNSUPPORTED;
    if (p->precision == SPH_PREC_DF64 &&
        (p->skf != 1 || (p->flags & (SPH_F_KERNEL_CORRECTION | SPH_F_ARTI_STRESS))))
        return SPH_E_UNSUPPORTED;
    if ((p->flags & SPH_F_KERNEL_CORRECTION) && p->precision != SPH_PREC_FP64) return SPH_E_UNSUPPORTED;
    // artificial heat: an FP64 pass B term of the SPH = 2 form without correction
    if ((p->flags & SPH_F_ARTI_HEAT) &&
        (p->precision != SPH_PREC_FP64 || p->pa_sph != 2 || (p->flags & SPH_F_KERNEL_CORRECTION)))
        return SPH_E_UNSUPPORTED;
    if (p->n_materials < 0 || p->n_materials > SPH_MAX_MATERIALS) return SPH_E_INVALID;
    if (!(p->dt > 0.0)) return SPH_E_INVALID;
    return SPH_OK;
}

// The model of an instance must match its batch: everything but dt, the
// material table, the spacing-tied lengths (wall_r0, contact_delta, as_dp)
// and the grid options is shared by all instances.
bool same_model(const sph_params& a, const sph_params& b) {
    return a.dim == b.dim && a.skf == b.skf && a.pa_sph == b.pa_sph && a.sle == b.sle && a.flags == b.flags &&
           a.precision == b.precision && a.gravity == b.gravity && a.av_alpha == b.av_alpha &&
           a.av_beta == b.av_beta && a.av_psi == b.av_psi && a.av_alpha_solid == b.av_alpha_solid &&
           a.av_beta_solid == b.av_beta_solid && a.cour_alpha == b.cour_alpha && a.cour_beta == b.cour_beta &&
           a.wall_fs == b.wall_fs && a.wall_p1 == b.wall_p1 && a.wall_p2 == b.wall_p2 &&
           a.pen_factor == b.pen_factor && a.pen_n1 == b.pen_n1 && a.pen_n2 == b.pen_n2 &&
           a.as_eps == b.as_eps && a.as_n == b.as_n && a.xsph_eps == b.xsph_eps;
}

// Parameter fields of the device view shared by every instance.
void fill_common(Dev& d, const sph_params& p) {
    d.dim = p.dim;
    d.d2 = p.dim * p.dim;
    d.tfs = sph::tf_stride_of(p.dim);
    d.precision = p.precision;
    d.skf = p.skf;
    d.pa_sph = p.pa_sph;
    d.sle = p.sle;
    d.flags = p.flags;
    d.scale_k = sph::scale_k_of(p.skf);
    d.gravity = p.gravity;
    d.av_alpha = p.av_alpha; d.av_beta = p.av_beta; d.av_psi = p.av_psi;
    d.av_alpha_solid = p.av_alpha_solid; d.av_beta_solid = p.av_beta_solid;
    d.av_psi_q = 0.25 * (p.av_psi * p.av_psi);
    d.av_alpha_h = -0.5 * p.av_alpha; d.av_alpha_h_solid = -0.5 * p.av_alpha_solid;
    d.cour_alpha = p.cour_alpha; d.cour_beta = p.cour_beta;
    d.wall_fs = p.wall_fs; d.wall_p1 = p.wall_p1; d.wall_p2 = p.wall_p2;
    d.pen_factor = p.pen_factor; d.pen_n1 = p.pen_n1; d.pen_n2 = p.pen_n2;
    d.wall_fs_f = (float)p.wall_fs; d.wall_p1_f = (float)p.wall_p1; d.wall_p2_f = (float)p.wall_p2;
    d.pen_factor_f = (float)p.pen_factor; d.pen_n1_f = (float)p.pen_n1; d.pen_n2_f = (float)p.pen_n2;
    d.as_eps = p.as_eps; d.as_n = p.as_n; d.xsph_eps = p.xsph_eps;
    d.av_alpha_f = (float)p.av_alpha; d.av_beta_f = (float)p.av_beta; d.av_psi_f = (float)p.av_psi;
    d.av_alpha_solid_f = (float)p.av_alpha_solid; d.av_beta_solid_f = (float)p.av_beta_solid;
    d.xsph_eps2_f = (float)p.xsph_eps * 2.0f;
    d.as_eps_f = (float)p.as_eps; d.as_n_f = (float)p.as_n;
}

void materials_of(const sph_params& p, sph::DevMaterial* out) {
    for (int k = 0; k < p.n_materials; ++k) {
        const sph_material& m = p.materials[k];
        sph::DevMaterial& o = out[k];
        o = sph::DevMaterial{};
        o.type = m.type; o.eos = m.eos; o.solid = m.solid; o.yield = m.yield;
        o.rho0 = m.rho0; o.c0 = m.c0; o.gamma = m.gamma; o.K = m.K; o.eta = m.eta;
        o.sigma_y = m.sigma_y; o.mg_cs = m.mg_cs; o.mg_s = m.mg_s;
        o.tait_b = m.gamma != 0.0 ? ((m.c0 * m.c0) * m.rho0) / m.gamma : 0.0;
        o.inv_rho0 = o.rho0 != 0.0 ? 1.0 / o.rho0 : 0.0;
        o.k_rho0 = o.rho0 != 0.0 ? o.K / o.rho0 : 0.0;
        o.rho0_f = (float)o.rho0; o.gamma_f = (float)o.gamma; o.eta_f = (float)o.eta;
        o.tait_b_f = (float)o.tait_b; o.k_rho0_f = o.rho0 != 0.0 ? (float)(o.K / o.rho0) : 0.0f;
        o.mg_cs_f = (float)o.mg_cs; o.mg_s_f = (float)o.mg_s;
    }
}

// Write instance k's table row and material rows to the device.
int push_instance(sph_ctx* ctx, int k) {
    HostInst& h = ctx->insts[k];
    sph::DevMaterial mats[SPH_MAX_MATERIALS] = {};
    materials_of(h.prm, mats);
    h.I.mat_base = k * SPH_MAX_MATERIALS;
    h.I.n_mat = h.prm.n_materials;
    h.I.wall_r0 = h.prm.wall_r0;
    h.I.contact_delta = h.prm.contact_delta;
    h.I.as_dp = h.prm.as_dp;
    h.I.ext_wall_r2 = (float)((h.prm.wall_r0 * 1.0001) * (h.prm.wall_r0 * 1.0001));
    h.I.ext_delta = (float)h.prm.contact_delta;
    h.I.wall_r0_f = (float)h.prm.wall_r0;
    CK(cudaMemcpyAsync(ctx->d_mat + (size_t)k * SPH_MAX_MATERIALS, mats, sizeof(mats), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->d.inst + k, &h.I, sizeof(sph::Inst), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// Pull the device-updated step counter and time of every instance.
int pull_instances(sph_ctx* ctx) {
    std::vector<sph::Inst> tab(ctx->max_inst);
    CK(cudaMemcpyAsync(tab.data(), ctx->d.inst, sizeof(sph::Inst) * ctx->max_inst, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < ctx->max_inst; ++k) {
        ctx->insts[k].I.step = tab[k].step;
        ctx->insts[k].I.time = tab[k].time;
    }
    return SPH_OK;
}

// FP32 mirrors of the mixed-precision passes (allocated on first use).
int ensure_mirrors(sph_ctx* ctx) {
    Dev& d = ctx->d;
    const int64_t N = ctx->capacity, D2 = (int64_t)ctx->prm.dim * ctx->prm.dim;
    int st = 0;
    if (ctx->prm.precision == SPH_PREC_DF64) {
        if (!d.pd0) {
            st |= dalloc(ctx, &d.pd0, N, ctx->allocs); st |= dalloc(ctx, &d.pd1, N, ctx->allocs);
            st |= dalloc(ctx, &d.vd0, N, ctx->allocs); st |= dalloc(ctx, &d.vd1, N, ctx->allocs);
            st |= dalloc(ctx, &d.ed0, N, ctx->allocs); st |= dalloc(ctx, &d.ed1, N, ctx->allocs);
            st |= dalloc(ctx, &d.ttd, N * D2, ctx->allocs);
            if (!st) {
                cudaMemsetAsync(d.ed1, 0, sizeof(float4) * N, ctx->stream);
                cudaMemsetAsync(d.ttd, 0, sizeof(float2) * N * D2, ctx->stream);
            }
        }
        return st ? SPH_E_NOMEM : SPH_OK;
    }
    if (!d.pr4) {
        st |= dalloc(ctx, &d.pr4, N, ctx->allocs); st |= dalloc(ctx, &d.vf4, N, ctx->allocs);
        st |= dalloc(ctx, &d.ef4, N, ctx->allocs); st |= dalloc(ctx, &d.pf4, N, ctx->allocs);
        st |= dalloc(ctx, &d.tf, N * d.tfs, ctx->allocs);
        if (!st) cudaMemsetAsync(d.tf, 0, sizeof(float) * N * d.tfs, ctx->stream);
    }
    if (d.has_solid && !d.sf) {
        st |= dalloc(ctx, &d.sf, N * d.tfs, ctx->allocs);
        st |= dalloc(ctx, &d.rf4, N, ctx->allocs);
        if (!st) {
            cudaMemsetAsync(d.sf, 0, sizeof(float) * N * d.tfs, ctx->stream);
            cudaMemsetAsync(d.rf4, 0, sizeof(float4) * N, ctx->stream);
        }
    }
    return st ? SPH_E_NOMEM : SPH_OK;
}

// Arrays of the optional per-step terms (summation density, XSPH), on first use.
int ensure_options(sph_ctx* ctx) {
    Dev& d = ctx->d;
    const int64_t N = ctx->capacity;
    const uint32_t F = ctx->prm.flags;
    int st = 0;
    if ((F & SPH_F_SUM_DENSITY) && !d.rsum) {
        st |= dalloc(ctx, &d.rsum, N, ctx->allocs);
        if (!st) cudaMemsetAsync(d.rsum, 0, sizeof(double) * N, ctx->stream);
    }
    if ((F & SPH_F_SUM_DENSITY) && (F & SPH_F_NORM_DENSITY) && !d.dxp) {
        st |= dalloc(ctx, &d.dxp, N, ctx->allocs);
        st |= dalloc(ctx, &d.dxp2, N, ctx->allocs);
        if (!st) {
            cudaMemsetAsync(d.dxp, 0, sizeof(double) * N, ctx->stream);
            cudaMemsetAsync(d.dxp2, 0, sizeof(double) * N, ctx->stream);
        }
    }
    if ((F & SPH_F_KERNEL_CORRECTION) && !d.kgc)
        st |= dalloc(ctx, &d.kgc, N * sph::KGC_STRIDE, ctx->allocs);
    if (ctx->prm.pa_sph == 3 && !d.pold) st |= dalloc(ctx, &d.pold, N, ctx->allocs);
    if (ctx->prm.pa_sph == 3 && !d.wraw) {
        st |= dalloc(ctx, &d.wraw, N, ctx->allocs);
        // contexts switched to SPH = 3 after their upload: the walls' current state
        if (!st && ctx->uploaded && ctx->d.n_wall > 0)
            sph::launch_wall_init(ctx->d, ctx->d.wall_off, ctx->d.n_wall, ctx->stream);
    }
    if ((F & SPH_F_AVER_VELOCITY) && !d.aver) {
        st |= dalloc(ctx, &d.aver, N, ctx->allocs);
        if (!st) cudaMemsetAsync(d.aver, 0, sizeof(double4) * N, ctx->stream);
    }
    return st ? fail(ctx, SPH_E_NOMEM, "summation-density / XSPH / kernel-correction arrays") : SPH_OK;
}

int ensure_solid(sph_ctx* ctx) {
    Dev& d = ctx->d;
    if (d.has_solid) return SPH_OK;
    const int64_t N = ctx->capacity, D2 = (int64_t)ctx->prm.dim * ctx->prm.dim;
    int st = 0;
    st |= dalloc(ctx, &d.shear, N * D2, ctx->allocs);
    st |= dalloc(ctx, &d.shear2, N * D2, ctx->allocs);
    st |= dalloc(ctx, &d.sig, N * D2, ctx->allocs);
    st |= dalloc(ctx, &d.dsdt, N * D2, ctx->allocs);
    st |= dalloc(ctx, &d.dsdt2, N * D2, ctx->allocs);
    st |= dalloc(ctx, &d.shear_prev, N * D2, ctx->allocs);
    st |= dalloc(ctx, &d.ras, N, ctx->allocs);
    if (st) return fail(ctx, SPH_E_NOMEM, "solid arrays");
    cudaMemsetAsync(d.sig, 0, sizeof(double) * N * D2, ctx->stream);
    cudaMemsetAsync(d.shear, 0, sizeof(double) * N * D2, ctx->stream);
    cudaMemsetAsync(d.shear2, 0, sizeof(double) * N * D2, ctx->stream);
    cudaMemsetAsync(d.ras, 0, sizeof(double4) * N, ctx->stream);
    d.has_solid = 1;
    if (ctx->prm.precision != SPH_PREC_FP64 && ensure_mirrors(ctx)) return fail(ctx, SPH_E_NOMEM, "mirrors");
    return SPH_OK;
}

// Cell arrays for `cells` cells (grows only).
int ensure_cells(sph_ctx* ctx, int64_t cells) {
    if (cells <= ctx->cell_cap) return SPH_OK;
    Dev& d = ctx->d;
    int64_t cap = std::max<int64_t>(cells, ctx->cell_cap * 3 / 2);
    int* fs = nullptr; int* ws = nullptr; int* cc = nullptr; uint32_t* sp = nullptr;
    std::vector<void*> fresh;
    int st = 0;
    st |= dalloc(ctx, &fs, cap + 2, fresh);
    st |= dalloc(ctx, &ws, cap + 2, fresh);
    st |= dalloc(ctx, &cc, cap + 2, fresh);
    st |= dalloc(ctx, &sp, sph::scan_partials(std::max<int64_t>(cap + 2, ctx->capacity * 256 / 4096 + 256)), fresh);
    if (st) { free_list(fresh); return fail(ctx, SPH_E_NOMEM, "cell arrays"); }
    if (d.wstart && ctx->cell_cap > 0)  // keep the wall starts of existing instances
        CK(cudaMemcpyAsync(ws, d.wstart, sizeof(int) * (ctx->cell_cap + 2), cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    free_list(ctx->grid_allocs);
    ctx->grid_allocs = fresh;
    d.fstart = fs; d.wstart = ws; d.ccount = cc; ctx->scan_part = sp;
    ctx->cell_cap = cap;
    return SPH_OK;
}

// Keys run up to total_cells + 1 (State == -1: total_cells; particles of a
// removed instance: total_cells + 1, so they sort last and are dropped).
void set_key_bits(sph_ctx* ctx) {
    ctx->key_bits = 1;
    while (((int64_t)1 << ctx->key_bits) <= (int64_t)ctx->d.total_cells + 1) ++ctx->key_bits;
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
    std::swap(d.pinst, d.pinst2);
    std::swap(d.shear, d.shear2);
    std::swap(d.dxp, d.dxp2);
}

// Cell keys, radix sort, cell starts and the reorder of the real particles
// (with the half kick when `kick`, for instances past their first step).
// Particles of removed instances sort to the end and are dropped.
int build_hash(sph_ctx* ctx, bool kick) {
    Dev& d = ctx->d;
    cudaStream_t s = ctx->stream;
    if (d.n_real == 0) { ctx->hash_valid = true; return SPH_OK; }
    CK(cudaMemsetAsync(d.ccount, 0, sizeof(int) * ((size_t)d.total_cells + 1), s));
    sph::launch_keys(d, d.n_real, d.xm, d.meta, d.pinst, d.keys, d.vals, d.ccount, s, true);
    // the cell starts need the counts alone: their scan runs beside the sort
    CK(cudaEventRecord(ctx->ev_keys, s));
    CK(cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_keys, 0));
    cudaError_t e = sph::sort_pairs(d.keys, d.vals, d.keys_s, d.vals_s, d.n_real, ctx->key_bits,
                                    ctx->sort_scratch, s, &ctx->launches);
    sph::exclusive_scan_u32((const uint32_t*)d.ccount, (uint32_t*)d.fstart, (int64_t)d.total_cells + 1,
                            ctx->scan_part, ctx->aux_stream, &ctx->launches);
    CK(cudaEventRecord(ctx->ev_scan, ctx->aux_stream));
    CK(cudaStreamWaitEvent(s, ctx->ev_scan, 0));
    if (e != cudaSuccess) return fail(ctx, SPH_E_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
    mark(ctx, 1);
    if (ctx->rest_pending) {
        CK(cudaStreamWaitEvent(s, ctx->ev_in, 0));
        sph::launch_host_state(d, 3, ctx->stage, s);
        ++ctx->launches;
        ctx->rest_pending = false;
    }
    sph::launch_permute(d, kick, s);
    swap_buffers(d);
    if (!kick) {
        std::swap(d.dvr, d.dvr2);
        std::swap(d.dedt, d.dedt2);
        std::swap(d.dsdt, d.dsdt2);
    }
    ctx->launches += 3;
    CK(cudaGetLastError());
    if (ctx->pending_remove) {
        d.n_real -= (int)ctx->pending_remove;
        ctx->pending_remove = 0;
    }
    ctx->hash_valid = true;
    ctx->density_done = false;
    ctx->kgc_done = false;
    return SPH_OK;
}

// kernelGradientCorrection of single_step (singleStep.f90:86), once per search.
int kgc_stage(sph_ctx* ctx) {
    if (!(ctx->d.flags & SPH_F_KERNEL_CORRECTION) || ctx->kgc_done) return SPH_OK;
    sph::launch_kernel_correction(ctx->d, ctx->stream);
    ctx->launches += 1;
    CK(cudaGetLastError());
    ctx->kgc_done = true;
    return SPH_OK;
}

// The density step of single_step (singleStep.f90:91-105), once per search:
// sum_density under SPH = 1 / 2 with summationDensity, con_density_riemann
// under SPH = 3 (whatever summationDensity says; con_density itself runs
// in pass A).
int density_stage(sph_ctx* ctx) {
    if (ctx->density_done) return SPH_OK;
    if (ctx->d.pa_sph == 3) {
        sph::launch_riemann_density(ctx->d, ctx->stream);
        ctx->launches += 1;
    } else if (ctx->d.flags & SPH_F_SUM_DENSITY) {
        sph::launch_density(ctx->d, ctx->stream);
        ctx->launches += 2;
    } else {
        return SPH_OK;
    }
    CK(cudaGetLastError());
    ctx->density_done = true;
    return SPH_OK;
}

int need(sph_ctx* ctx, bool hash) {
    if (!ctx) return SPH_E_INVALID;
    if (!ctx->uploaded) return fail(ctx, SPH_E_STATE, "no particles uploaded");
    if (hash && !ctx->hash_valid) return fail(ctx, SPH_E_STATE, "call sph_nnps first");
    return SPH_OK;
}

// Entry points whose arrays run over one system's upload order: the systems
// of a batch share those indices, so a batch reads them per instance.
int need_plain(sph_ctx* ctx, bool hash) {
    int st = need(ctx, hash);
    if (st) return st;
    if (ctx->batch) return fail(ctx, SPH_E_UNSUPPORTED, "per-system arrays of a batch: use sph_batch_get_field");
    return SPH_OK;
}

int gather_to_host(sph_ctx* ctx, int field, double* out, int64_t count, int inst = -1) {
    if (!out) return SPH_OK;
    sph::launch_gather_field(ctx->d, field, ctx->stage, inst, ctx->stream);
    ++ctx->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, ctx->stage, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int comps_of(const Dev& d, int field) {
    switch (field) {
    case SPH_FIELD_X: case SPH_FIELD_V: case SPH_FIELD_DISP: case SPH_FIELD_DVDT: case SPH_FIELD_AVER: return d.dim;
    case SPH_FIELD_STRESS: case SPH_FIELD_SHEAR: case SPH_FIELD_DSDT: case SPH_FIELD_STRAIN: return d.d2;
    default: return 1;
    }
}

int check_status_word(sph_ctx* ctx) {
    uint32_t st = 0;
    CK(cudaMemcpyAsync(&st, ctx->d.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st & sph::ST_NONFINITE) return fail(ctx, SPH_E_NONFINITE, "non-finite rho, v, e or x after a step");
    if (st & sph::ST_H_RANGE)
        return fail(ctx, SPH_E_RANGE, "an evolved smoothing length outgrew the hash cell; set sph_params.cell_size "
                                      "to scale_k times the largest h expected");
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
    mark(ctx, 0);
    int st = build_hash(ctx, true);
    if (st) return st;
    if ((st = kgc_stage(ctx))) return st;
    if ((st = density_stage(ctx))) return st;
    st = run_passes(ctx, sph::step_terms(d), true, false);
    if (st) return st;
    sph::launch_update(d, ctx->stream);
    ctx->launches += (d.n_real > 0 ? 1 : 0) + (d.n_inst > 0 ? 1 : 0);
    mark(ctx, 5);
    CK(cudaGetLastError());
    if (ctx->timing && ++ctx->ev_used == sph_ctx::kPool) flush_timing(ctx);
    ctx->step += 1;
    ctx->time += ctx->insts[0].prm.dt;
    ctx->hash_valid = false;
    return SPH_OK;
}

// The multiply-shift reciprocals of nc[0] and nc[1] (Grid::div_m, div_l):
// l = ceil(log2 nc), m = ceil(2^(31 + l) / nc), so that n / nc equals
// (n m) >> (31 + l) for every 0 <= n < 2^31.
void grid_divisors(const sph::Grid& g, unsigned long long m[2], int l[2]) {
    for (int a = 0; a < 2; ++a) {
        const uint64_t dv = (uint64_t)std::max(g.nc[a], 1);
        int k = 0;
        while ((1ull << k) < dv) ++k;
        l[a] = k;
        m[a] = ((1ull << (31 + k)) + dv - 1) / dv;
    }
}

// Grid of one instance from its particles and options (include/sph_gpu.h:
// cell size scale_k * max h, domain = bounding box + margin or the given box).
int make_grid_bounds(sph_ctx* ctx, const sph_params& P, const double* lo, const double* hi, double hmin,
                     double hmax, sph::Grid* out);

int make_grid(sph_ctx* ctx, const sph_params& P, int64_t N, const double* x, const double* h,
              sph::Grid* out) {
    const int dim = P.dim;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, hmax = 0.0, hmin = 1e300;
    for (int a = 0; a < dim; ++a) { lo[a] = 1e300; hi[a] = -1e300; }
    for (int64_t i = 0; i < N; ++i) {
        for (int a = 0; a < dim; ++a) {
            double xv = x[i * dim + a];
            if (!std::isfinite(xv)) return fail(ctx, SPH_E_INVALID, "non-finite position");
            lo[a] = std::min(lo[a], xv);
            hi[a] = std::max(hi[a], xv);
        }
        if (!(h[i] > 0.0) || !std::isfinite(h[i])) return fail(ctx, SPH_E_INVALID, "smoothing length must be > 0");
        hmax = std::max(hmax, h[i]);
        hmin = std::min(hmin, h[i]);
    }
    return make_grid_bounds(ctx, P, lo, hi, hmin, hmax, out);
}

// Grid from the particles' bounding box [lo, hi] and smoothing-length range.
int make_grid_bounds(sph_ctx* ctx, const sph_params& P, const double* lo, const double* hi, double hmin,
                     double hmax, sph::Grid* out) {
    const int dim = P.dim;
    const double reach_max = hmax * sph::scale_k_of(P.skf);
    double cs = P.cell_size > 0.0 ? P.cell_size : reach_max * (1.0 + 1e-9);
    if (cs < reach_max) return fail(ctx, SPH_E_INVALID, "cell_size below scale_k * max(h)");
    bool user_domain = true;
    for (int a = 0; a < dim; ++a)
        if (!(P.domain_lo[a] < P.domain_hi[a])) user_domain = false;
    const double margin = P.grid_margin > 0.0 ? P.grid_margin : 2.0 * cs;
    sph::Grid g{};
    int64_t ncells = 1;
    for (;;) {
        ncells = 1;
        for (int a = 0; a < 3; ++a) {
            if (a >= dim) { g.lo[a] = 0.0; g.nc[a] = 1; continue; }
            double l = user_domain ? P.domain_lo[a] : lo[a] - margin;
            double u = user_domain ? P.domain_hi[a] : hi[a] + margin;
            g.lo[a] = l;
            int64_t nc = std::max<int64_t>((int64_t)std::ceil((u - l) / cs), 1);
            g.nc[a] = (int)std::min<int64_t>(nc, 1 << 24);
            ncells *= g.nc[a];
        }
        if (ncells <= (int64_t)16 * 1024 * 1024 - 2) break;
        cs *= 1.25;  // very sparse domains: coarser cells (still exact)
    }
    g.cs = cs;
    g.inv_cs = 1.0 / cs;
    g.cs_f = (float)cs;
    grid_divisors(g, g.div_m, g.div_l);
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
    *out = g;
    return SPH_OK;
}

// Upload one instance: its real particles to slots [d.n_real, +n_r), its
// walls to [ctx->wall_end, +n_w) in cell order, its grid appended to the cell
// space, its table and material rows to the device.
// Generated blocks of one instance (sph_upload_blocks / sph_batch_add_blocks).
struct BlockSource {
    const sph_block* blocks = nullptr;
    int n = 0, n_real = 0;
};

int64_t block_count(const sph_block& b, int dim) {
    int64_t c = 1;
    for (int a = 0; a < 3; ++a) c *= (a < dim) ? (int64_t)b.n[a] : 1;
    return c;
}

// Check the blocks and count their real and wall particles.
int check_blocks(sph_ctx* ctx, int dim, int32_t nb, const sph_block* blocks, int32_t nrb, int64_t* n_r,
                 int64_t* n_w) {
    if (!blocks || nb <= 0 || nb > 1024 || nrb < 1 || nrb > nb) return fail(ctx, SPH_E_INVALID, "bad block list");
    *n_r = *n_w = 0;
    for (int b = 0; b < nb; ++b) {
        const sph_block& B = blocks[b];
        for (int a = 0; a < 3; ++a)
            if ((a < dim && B.n[a] < 1) || (a >= dim && B.n[a] > 1) || !std::isfinite(B.origin[a]) ||
                !std::isfinite(B.spacing[a]))
                return fail(ctx, SPH_E_INVALID, "block lattice");
        if (!(B.h > 0.0) || !std::isfinite(B.mass) || !std::isfinite(B.c))
            return fail(ctx, SPH_E_INVALID, "block fields");
        if (B.tait_b > 0.0 ? !(B.tait_gamma > 0.0 && B.tait_rho0 > 0.0) : !(B.rho > 0.0))
            return fail(ctx, SPH_E_INVALID, "density must be > 0");
        if (B.up_axis < 0 || B.up_axis >= dim) return fail(ctx, SPH_E_INVALID, "block up_axis");
        if (B.clamp_axis < 0 || B.clamp_axis >= dim) return fail(ctx, SPH_E_INVALID, "block clamp_axis");
        const int64_t c = block_count(B, dim);
        (b < nrb ? *n_r : *n_w) += c;
    }
    return SPH_OK;
}

int add_instance(sph_ctx* ctx, int k, const sph_params& P, int64_t n_r, int64_t n_w, const double* x,
                 const double* v, const double* mass, const double* rho, const double* p, const double* e,
                 const double* c, const double* h, const int32_t* type, const int32_t* state,
                 const int32_t* boundary, const double* shear, const BlockSource& gen = BlockSource{}) {
    Dev& d = ctx->d;
    const int dim = ctx->prm.dim, D2 = dim * dim;
    const int64_t N = n_r + n_w;
    bool solid = false;
    const bool kgc = ctx->prm.flags & SPH_F_KERNEL_CORRECTION;
    const char* kgc_msg = "kernel correction needs every real particle to be a solid "
                          "(Type > 100): for other targets the reference's solve divides 0 by 0";
    sph::Grid g{};
    int st;
    if (gen.blocks) {
        double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, hmin = 1e300, hmax = 0.0;
        for (int a = 0; a < dim; ++a) { lo[a] = 1e300; hi[a] = -1e300; }
        for (int b = 0; b < gen.n; ++b) {
            const sph_block& B = gen.blocks[b];
            if (std::abs(B.type) > 100) solid = true;
            if (kgc && b < gen.n_real && B.type <= 100) return fail(ctx, SPH_E_UNSUPPORTED, kgc_msg);
            for (int a = 0; a < dim; ++a) {
                const double x0 = B.origin[a] + 0.5 * B.spacing[a];
                const double x1 = B.origin[a] + (B.n[a] - 0.5) * B.spacing[a];
                lo[a] = std::min(lo[a], std::min(x0, x1));
                hi[a] = std::max(hi[a], std::max(x0, x1));
            }
            hmin = std::min(hmin, B.h);
            hmax = std::max(hmax, B.h);
        }
        st = make_grid_bounds(ctx, P, lo, hi, hmin, hmax, &g);
    } else {
        for (int64_t i = 0; i < N; ++i) {
            if (!(rho[i] > 0.0)) return fail(ctx, SPH_E_INVALID, "density must be > 0");
            if (std::abs(type[i]) > 100) solid = true;
        }
        if (kgc)
            for (int64_t i = 0; i < n_r; ++i)
                if (type[i] <= 100) return fail(ctx, SPH_E_UNSUPPORTED, kgc_msg);
        st = make_grid(ctx, P, N, x, h, &g);
    }
    if (st) return st;
    if (solid && ctx->prm.precision == SPH_PREC_DF64)
        return fail(ctx, SPH_E_UNSUPPORTED, "the DF64 pair passes cover fluid systems only");
    if (solid && (st = ensure_solid(ctx))) return st;
    if (ctx->prm.precision != SPH_PREC_FP64 && ensure_mirrors(ctx)) return fail(ctx, SPH_E_NOMEM, "FP32 mirrors");
    if (!d.strain && dalloc(ctx, &d.strain, ctx->capacity * D2, ctx->allocs)) return fail(ctx, SPH_E_NOMEM, "strain");
    const int64_t base = d.total_cells;
    if (base + (int64_t)g.ncells + 2 >= ((int64_t)1 << 31))
        return fail(ctx, SPH_E_RANGE, "the systems' cell grids exceed 2^31 cells in total");
    if ((st = ensure_cells(ctx, base + g.ncells + 1))) return st;

    HostInst& hi = ctx->insts[k];
    hi = HostInst{};
    hi.used = true;
    hi.prm = P;
    hi.n_real = n_r;
    hi.n_wall = n_w;
    hi.wall_first = ctx->wall_end;
    hi.I.grid = g;
    hi.I.cell_base = (int)base;
    hi.I.n_real = (int)n_r;
    hi.I.wall_first = (int)ctx->wall_end;
    hi.I.n_wall = (int)n_w;
    hi.I.step = 0;
    hi.I.active = 1;
    hi.I.dt = P.dt;
    hi.I.time = 0.0;
    if ((st = push_instance(ctx, k))) return st;

    // host -> device staging (x, v, m, rho, p, e, c, h, shear | type, state, bnd),
    // freed before returning (not counted in device_bytes)
    const int64_t db0 = ctx->device_bytes;
    std::vector<void*> tmp;
    double *dx_ = nullptr, *dv_ = nullptr, *dsc = nullptr, *dsh = nullptr;
    int* dt_ = nullptr;
    uint32_t* word = nullptr;
    st = 0;
    st |= dalloc(ctx, &dx_, N * dim, tmp);
    st |= dalloc(ctx, &dv_, N * dim, tmp);
    st |= dalloc(ctx, &dsc, N * 6, tmp);
    st |= dalloc(ctx, &dt_, N * 3, tmp);
    if (shear && d.has_solid) st |= dalloc(ctx, &dsh, N * D2, tmp);
    st |= dalloc(ctx, &word, N * 2 + 2, tmp);
    if (st) { free_list(tmp); ctx->device_bytes = db0; return fail(ctx, SPH_E_NOMEM, "upload staging"); }
    cudaStream_t s = ctx->stream;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
    };
    const int real_dst = d.n_real;
    const int wall_dst = (int)ctx->wall_end;
    uint32_t* worder = word;
    uint32_t* wkeys = word + N + 1;
    std::vector<uint32_t> iota(gen.blocks ? 1 : std::max<int64_t>(n_w, 1));
    for (int64_t q = 0; !gen.blocks && q < n_w; ++q) iota[q] = (uint32_t)q;
    cudaError_t ce = cudaSuccess;
#define UP(dst, src, bytes) do { ce = up(dst, src, bytes); if (ce) goto cuda_fail; } while (0)
    if (gen.blocks) {
        // the block table and its particle offsets, then one generation launch
        sph_block* db = nullptr;
        int64_t* dstart = nullptr;
        if (dalloc(ctx, &db, gen.n, tmp) || dalloc(ctx, &dstart, gen.n + 1, tmp)) {
            free_list(tmp); ctx->device_bytes = db0; return fail(ctx, SPH_E_NOMEM, "block table");
        }
        std::vector<int64_t> starts(gen.n + 1, 0);
        for (int b = 0; b < gen.n; ++b) starts[b + 1] = starts[b] + block_count(gen.blocks[b], dim);
        UP(db, gen.blocks, sizeof(sph_block) * gen.n);
        UP(dstart, starts.data(), sizeof(int64_t) * (gen.n + 1));
        ce = cudaStreamSynchronize(s); if (ce) goto cuda_fail;  // the host vectors go out of scope
        sph::launch_generate_blocks(db, dstart, gen.n, dim, N, n_r, dx_, dv_, dsc, dt_, worder, s);
        ++ctx->launches;
        if (dsh) { ce = cudaMemsetAsync(dsh, 0, sizeof(double) * N * D2, s); if (ce) goto cuda_fail; }
    } else {
        UP(dx_, x, sizeof(double) * N * dim);
        UP(dv_, v, sizeof(double) * N * dim);
        UP(dsc + 0 * N, mass, sizeof(double) * N);
        UP(dsc + 1 * N, rho, sizeof(double) * N);
        UP(dsc + 2 * N, p, sizeof(double) * N);
        UP(dsc + 3 * N, e, sizeof(double) * N);
        UP(dsc + 4 * N, c, sizeof(double) * N);
        UP(dsc + 5 * N, h, sizeof(double) * N);
        UP(dt_, type, sizeof(int) * N);
        if (state) UP(dt_ + N, state, sizeof(int) * N);
        if (boundary) UP(dt_ + 2 * N, boundary, sizeof(int) * N);
        if (dsh) UP(dsh, shear, sizeof(double) * N * D2);
        if (n_w > 0) UP(worder, iota.data(), sizeof(uint32_t) * n_w);
    }
#undef UP
    {
        ce = cudaStreamSynchronize(s); if (ce) goto cuda_fail;
        // the instance's particles are live in the counts that follow
        d.n_real = real_dst + (int)n_r;
        d.n_wall = (int)(ctx->wall_end - d.wall_off) + (int)n_w;
        d.total_cells = (int)(base + g.ncells);
        set_key_bits(ctx);
        // 1) pack with identity wall order
        sph::launch_pack_upload(d, (int)n_r, (int)n_w, real_dst, wall_dst, k, dx_, dv_, dsc, dsc + N, dsc + 2 * N,
                                dsc + 3 * N, dsc + 4 * N, dsc + 5 * N, dt_, (state || gen.blocks) ? dt_ + N : nullptr,
                                (boundary || gen.blocks) ? dt_ + 2 * N : nullptr, dsh, worder, s);
        ++ctx->launches;
        // 2) wall keys -> sort -> wall order; wall cell starts of this instance
        ce = cudaMemsetAsync(d.ccount + base, 0, sizeof(int) * ((size_t)g.ncells + 1), s); if (ce) goto cuda_fail;
        if (n_w > 0) {
            sph::launch_keys(d, (int)n_w, d.xm + wall_dst, d.meta + wall_dst, d.pinst + wall_dst, d.keys, d.vals,
                             d.ccount, s, false);
            ce = sph::sort_pairs(d.keys, d.vals, wkeys, worder, n_w, ctx->key_bits, ctx->sort_scratch, s,
                                 &ctx->launches);
            if (ce) goto cuda_fail;
            ++ctx->launches;
        }
        sph::exclusive_scan_u32((const uint32_t*)d.ccount + base, (uint32_t*)d.wstart + base, g.ncells + 1,
                                ctx->scan_part, s, &ctx->launches);
        sph::launch_add_offset(d.wstart + base, g.ncells + 1, wall_dst - d.wall_off, s);
        // 3) pack again with the walls in cell order, wall EOS
        sph::launch_pack_upload(d, (int)n_r, (int)n_w, real_dst, wall_dst, k, dx_, dv_, dsc, dsc + N, dsc + 2 * N,
                                dsc + 3 * N, dsc + 4 * N, dsc + 5 * N, dt_, (state || gen.blocks) ? dt_ + N : nullptr,
                                (boundary || gen.blocks) ? dt_ + 2 * N : nullptr, dsh, worder, s);
        sph::launch_wall_init(d, wall_dst, (int)n_w, s);
        sph::launch_kref(d, k, n_r > 0 ? (int)real_dst : -1, s);
        ctx->launches += 4;
        ce = cudaMemsetAsync(d.cres + 3 * k, 0, 3 * sizeof(double), s); if (ce) goto cuda_fail;
        ce = cudaMemsetAsync(d.cmax + k, 0, sizeof(unsigned long long), s); if (ce) goto cuda_fail;
        ce = cudaGetLastError(); if (ce) goto cuda_fail;
        ce = cudaStreamSynchronize(s); if (ce) goto cuda_fail;
    }
    free_list(tmp);
    ctx->device_bytes = db0;
    ctx->wall_end += n_w;
    ctx->uploaded = true;
    ctx->hash_valid = false;
    return SPH_OK;
cuda_fail:
    cudaStreamSynchronize(s);
    free_list(tmp);
    ctx->device_bytes = db0;
    return fail(ctx, SPH_E_CUDA, std::string("upload: ") + cudaGetErrorString(ce));
}

// The context's streams and events (each after its work has ended).
void destroy_streams(sph_ctx* ctx) {
    for (cudaStream_t* st : {&ctx->in_stream, &ctx->aux_stream}) {
        if (*st) {
            cudaStreamSynchronize(*st);
            cudaStreamDestroy(*st);
            *st = nullptr;
        }
    }
    for (cudaEvent_t* e : {&ctx->ev_x, &ctx->ev_in, &ctx->ev_keys, &ctx->ev_scan}) {
        if (*e) cudaEventDestroy(*e);
        *e = nullptr;
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = nullptr;
}

// Allocation of a context with `slots` particle slots and `max_inst` instances.
int create_ctx(const sph_params* prm, int max_inst, int64_t slots, sph_ctx** out) {
    sph_ctx* ctx = new sph_ctx();
    ctx->prm = *prm;
    ctx->capacity = slots;
    ctx->max_inst = max_inst;
    ctx->insts.resize(max_inst);
    cudaGetDevice(&ctx->device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return SPH_E_CUDA;
    }
    if (cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_keys, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_scan, cudaEventDisableTiming) != cudaSuccess) {
        destroy_streams(ctx);
        delete ctx;
        return SPH_E_CUDA;
    }
    fill_common(ctx->d, *prm);
    Dev& d = ctx->d;
    const int64_t N = slots;
    const int64_t D2 = (int64_t)prm->dim * prm->dim;
    auto& L = ctx->allocs;
    int st = 0;
    st |= dalloc(ctx, &d.xm, N, L); st |= dalloc(ctx, &d.vr, N, L); st |= dalloc(ctx, &d.eh, N, L);
    st |= dalloc(ctx, &d.dsp, N, L); st |= dalloc(ctx, &d.meta, N, L); st |= dalloc(ctx, &d.pinst, N, L);
    st |= dalloc(ctx, &d.xm2, N, L); st |= dalloc(ctx, &d.vr2, N, L); st |= dalloc(ctx, &d.eh2, N, L);
    st |= dalloc(ctx, &d.dsp2, N, L); st |= dalloc(ctx, &d.meta2, N, L); st |= dalloc(ctx, &d.pinst2, N, L);
    st |= dalloc(ctx, &d.posf, N, L); st |= dalloc(ctx, &d.pa4, N, L); st |= dalloc(ctx, &d.tt, N * D2, L);
    st |= dalloc(ctx, &d.dvr, N, L); st |= dalloc(ctx, &d.dedt, N, L); st |= dalloc(ctx, &d.tds, N, L);
    st |= dalloc(ctx, &d.dvr2, N, L); st |= dalloc(ctx, &d.dedt2, N, L);
    st |= dalloc(ctx, &d.prev_vr, N, L); st |= dalloc(ctx, &d.prev_e, N, L);
    st |= dalloc(ctx, &d.keys, N, L); st |= dalloc(ctx, &d.vals, N, L);
    st |= dalloc(ctx, &d.keys_s, N, L); st |= dalloc(ctx, &d.vals_s, N, L);
    st |= dalloc(ctx, &d.nneigh, N, L);
    st |= dalloc(ctx, &d.status, 1, L);
    st |= dalloc(ctx, &d.inst, max_inst, L);
    st |= dalloc(ctx, &ctx->d_mat, (int64_t)max_inst * SPH_MAX_MATERIALS, L);
    st |= dalloc(ctx, &d.cmax, max_inst, L);
    st |= dalloc(ctx, &d.cpart, (N + 255) / 256, L);
    st |= dalloc(ctx, &d.cpinst, (N + 255) / 256, L);
    st |= dalloc(ctx, &d.cnp, N, L);
    st |= dalloc(ctx, &d.cres, 3 * max_inst, L);
    sph::KRef* kref = nullptr;
    st |= dalloc(ctx, &kref, max_inst, L);
    d.kref = kref;
    st |= dalloc(ctx, &ctx->d_counts, N, L);
    st |= dalloc(ctx, &ctx->d_offsets, N + 1, L);
    ctx->stage_bytes = sizeof(double) * N * std::max<int64_t>(D2, 2 * prm->dim + 2) + 64;
    st |= dalloc(ctx, (char**)&ctx->stage, ctx->stage_bytes, L);
    ctx->sort_scratch_bytes = sph::sort_scratch_bytes(N, 32);
    st |= dalloc(ctx, (char**)&ctx->sort_scratch, ctx->sort_scratch_bytes, L);
    if (st) {
        free_list(ctx->allocs);
        destroy_streams(ctx);
        delete ctx;
        return SPH_E_NOMEM;
    }
    d.mat = ctx->d_mat;
    d.n_inst = max_inst;
    d.tile_tpb = 128;
    d.persistent = 0;
    d.lane_shift = 0;
    d.tile_k = sph::default_tile_k(prm->dim);
    cudaMemsetAsync(d.status, 0, sizeof(uint32_t), ctx->stream);
    cudaMemsetAsync(d.inst, 0, sizeof(sph::Inst) * max_inst, ctx->stream);
    cudaMemsetAsync(d.cmax, 0, sizeof(unsigned long long) * max_inst, ctx->stream);
    cudaMemsetAsync(d.cres, 0, sizeof(double) * 3 * max_inst, ctx->stream);
    cudaMemsetAsync((void*)d.kref, 0, sizeof(sph::KRef) * max_inst, ctx->stream);   // h = +0: no reference
    if ((prm->precision != SPH_PREC_FP64 && ensure_mirrors(ctx) != SPH_OK) || ensure_options(ctx) != SPH_OK) {
        free_list(ctx->allocs);
        destroy_streams(ctx);
        delete ctx;
        return SPH_E_NOMEM;
    }
    cudaStreamSynchronize(ctx->stream);
    ctx->ev.resize((size_t)sph_ctx::kPool * (SPH_NUM_STAGES + 1));
    for (auto& e2 : ctx->ev) cudaEventCreate(&e2);
    *out = ctx;
    return SPH_OK;
}

void drop_graph(sph_ctx* ctx) {
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
}

// Capture two steps (an even number, so the double buffers end where they
// started) into a graph; valid while the particle counts and cell space stay.
int capture_graph(sph_ctx* ctx) {
    drop_graph(ctx);
    const bool timing = ctx->timing;
    ctx->timing = false;
    const int64_t l0 = ctx->launches, s0 = ctx->step;
    const double t0 = ctx->time;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int st = one_step(ctx);
    if (!st) st = one_step(ctx);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->timing = timing;
    ctx->step = s0;
    ctx->time = t0;
    if (st) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return fail(ctx, SPH_E_CUDA, "graph capture"); }
    e = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { ctx->graph = nullptr; return fail(ctx, SPH_E_CUDA, "graph instantiate"); }
    ctx->graph_launches = ctx->launches - l0;
    ctx->launches = l0;
    ctx->graph_key_bits = ctx->key_bits;
    ctx->graph_n_real = ctx->d.n_real;
    ctx->graph_cells = ctx->d.total_cells;
    ctx->graph_xm = ctx->d.xm;
    ctx->graph_dvr = ctx->d.dvr;
    return SPH_OK;
}

// The graph's kernel arguments hold buffer pointers: it replays only from the
// buffer parity, counts and cell space it was captured with.
bool graph_usable(sph_ctx* ctx) {
    return ctx->graph && ctx->graph_n_real == ctx->d.n_real && ctx->graph_cells == ctx->d.total_cells &&
           ctx->graph_key_bits == ctx->key_bits && ctx->pending_remove == 0 &&
           ctx->graph_xm == (const void*)ctx->d.xm && ctx->graph_dvr == (const void*)ctx->d.dvr;
}

// nsteps leap-frog steps: eager launches, or graph replays of two steps once
// every system is past its first step (the graph holds no host decisions).
// From three steps on a call captures (or reuses) the graph, so that a
// three-step warm-up from the initial state leaves it captured.
int advance_steps(sph_ctx* ctx, int64_t nsteps) {
    int st;
    int64_t k = 0;
    const bool graphs = ctx->use_graphs && !ctx->timing && nsteps >= 3;
    if (graphs) {
        // first steps (no kick) and removals run eagerly
        while (k < nsteps && (ctx->step == 0 || ctx->pending_remove)) {
            if ((st = one_step(ctx))) return st;
            ++k;
        }
        if (nsteps - k >= 2) {
            if (!graph_usable(ctx) && (st = capture_graph(ctx))) return st;
            for (; k + 2 <= nsteps; k += 2) {
                CK(cudaGraphLaunch(ctx->graph, ctx->stream));
                ctx->launches += ctx->graph_launches;
                ctx->step += 2;
                ctx->time += 2 * ctx->insts[0].prm.dt;
            }
            ctx->hash_valid = false;
        }
    }
    for (; k < nsteps; ++k)
        if ((st = one_step(ctx))) return st;
    return SPH_OK;
}

int inst_index(sph_ctx* ctx, int32_t inst) {
    if (!ctx) return SPH_E_INVALID;
    if (inst < 0 || inst >= ctx->max_inst || !ctx->insts[inst].used || !ctx->insts[inst].I.active)
        return fail(ctx, SPH_E_INVALID, "no such instance");
    return SPH_OK;
}

// ---- state snapshots (sph_state_save / sph_state_load) --------------------
// A snapshot is a header, the host records of the instances and the live
// ranges of the device arrays that carry state from one step to the next:
// particle state and the last step's rates (the next half kick reads them),
// the once-written wall data (positions, FP32 mirrors, pressure, wall cell
// starts), the instance and material tables and the Courant statistics.
// Arrays that every step rewrites before reading (cell starts of the real
// particles, pair-pass outputs, sort scratch, second buffers) are not saved.
struct StateHeader {
    char magic[8];
    uint32_t version, header_bytes;
    uint32_t params_bytes, inst_bytes, material_bytes, reserved;
    sph_params prm;
    int32_t batch, max_inst, has_solid, mirrors, dxp, key_bits;
    int64_t capacity, real_cap, wall_end, cell_cap, pending_remove;
    int64_t n_real, n_wall, wall_off, total_cells, step;
    double time;
    int64_t payload_bytes;
};
struct StateInst {
    sph::Inst I;
    sph_params prm;
    int64_t n_real, n_wall, wall_first;
    int32_t used, reserved;
};
constexpr char kStateMagic[8] = {'S', 'P', 'H', 'S', 'T', 'A', 'T', 'E'};
constexpr uint32_t kStateVersion = 4;

struct StateArray {
    void* ptr;
    size_t bytes_per_item;  // per particle, or per item of a table
    int64_t items;          // 0 for particle arrays (live ranges)
    void* twin = nullptr;   // second buffer of double-buffered state: walls live in both
};

std::vector<StateArray> state_arrays(sph_ctx* ctx) {
    Dev& d = ctx->d;
    const size_t D2 = (size_t)ctx->prm.dim * ctx->prm.dim;
    std::vector<StateArray> a = {
        {d.xm, sizeof(double4), 0, d.xm2}, {d.vr, sizeof(double4), 0, d.vr2}, {d.eh, sizeof(double4), 0, d.eh2},
        {d.dsp, sizeof(double4), 0, d.dsp2}, {d.meta, sizeof(int4), 0, d.meta2}, {d.pinst, sizeof(int), 0, d.pinst2},
        {d.posf, sizeof(float4), 0}, {d.pa4, sizeof(double4), 0}, {d.tt, sizeof(double) * D2, 0},
        {d.dvr, sizeof(double4), 0}, {d.dedt, sizeof(double), 0},
    };
    if (d.has_solid) {
        a.push_back({d.shear, sizeof(double) * D2, 0, d.shear2});
        a.push_back({d.sig, sizeof(double) * D2, 0});
        a.push_back({d.dsdt, sizeof(double) * D2, 0});
        a.push_back({d.ras, sizeof(double4), 0});
    }
    if (d.pr4) {
        a.push_back({d.pr4, sizeof(float4), 0});
        a.push_back({d.vf4, sizeof(float4), 0});
        a.push_back({d.ef4, sizeof(float4), 0});
        a.push_back({d.pf4, sizeof(float4), 0});
        a.push_back({d.tf, sizeof(float) * d.tfs, 0});
    }
    if (d.sf) {
        a.push_back({d.sf, sizeof(float) * d.tfs, 0});
        a.push_back({d.rf4, sizeof(float4), 0});
    }
    if (d.dxp) a.push_back({d.dxp, sizeof(double), 0});
    if (d.wraw) a.push_back({d.wraw, sizeof(double2), 0});
    a.push_back({d.wstart, sizeof(int), ctx->cell_cap + 2});
    a.push_back({d.inst, sizeof(sph::Inst), ctx->max_inst});
    a.push_back({ctx->d_mat, sizeof(sph::DevMaterial), (int64_t)ctx->max_inst * SPH_MAX_MATERIALS});
    a.push_back({d.cres, sizeof(double), 3 * (int64_t)ctx->max_inst});
    a.push_back({(void*)d.kref, sizeof(sph::KRef), (int64_t)ctx->max_inst});
    return a;
}

// Live particle ranges: real slots [0, n_real) and wall slots [wall_off, wall_end).
int64_t state_particles(const sph_ctx* ctx) {
    return (int64_t)ctx->d.n_real + (ctx->wall_end - ctx->d.wall_off);
}

int64_t state_payload(sph_ctx* ctx) {
    int64_t b = (int64_t)sizeof(StateInst) * ctx->max_inst;
    const int64_t np = state_particles(ctx);
    for (const auto& x : state_arrays(ctx)) b += (int64_t)x.bytes_per_item * (x.items ? x.items : np);
    return b;
}

// Copy every saved array between the device and `buf` (to_host: save).
int state_copy(sph_ctx* ctx, unsigned char* buf, bool to_host) {
    const int64_t nr = ctx->d.n_real, w0 = ctx->d.wall_off, nw = ctx->wall_end - ctx->d.wall_off;
    const auto kind = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
    for (const auto& x : state_arrays(ctx)) {
        unsigned char* dev = (unsigned char*)x.ptr;
        if (x.items) {
            const size_t n = x.bytes_per_item * (size_t)x.items;
            CK(to_host ? cudaMemcpyAsync(buf, dev, n, kind, ctx->stream) : cudaMemcpyAsync(dev, buf, n, kind, ctx->stream));
            buf += n;
            continue;
        }
        const size_t r = x.bytes_per_item * (size_t)nr, w = x.bytes_per_item * (size_t)nw;
        unsigned char* wdev = dev + x.bytes_per_item * (size_t)w0;
        if (r) CK(to_host ? cudaMemcpyAsync(buf, dev, r, kind, ctx->stream) : cudaMemcpyAsync(dev, buf, r, kind, ctx->stream));
        buf += r;
        if (w) CK(to_host ? cudaMemcpyAsync(buf, wdev, w, kind, ctx->stream) : cudaMemcpyAsync(wdev, buf, w, kind, ctx->stream));
        if (w && !to_host && x.twin)  // the walls of the other buffer
            CK(cudaMemcpyAsync((unsigned char*)x.twin + x.bytes_per_item * (size_t)w0, buf, w, kind, ctx->stream));
        buf += w;
    }
    CK(cudaStreamSynchronize(ctx->stream));
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
    st = create_ctx(prm, 1, capacity, out);
    if (st == SPH_OK) (*out)->insts[0].prm = *prm;
    return st;
}

int sph_destroy(sph_ctx* ctx) {
    if (!ctx) return SPH_E_INVALID;
    cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    if (ctx->d_list) cudaFree(ctx->d_list);
    free_list(ctx->allocs);
    free_list(ctx->grid_allocs);
    for (auto& e2 : ctx->ev)
        if (e2) cudaEventDestroy(e2);
    destroy_streams(ctx);
    delete ctx;
    return SPH_OK;
}

int sph_set_params(sph_ctx* ctx, const sph_params* prm) {
    if (!ctx) return SPH_E_INVALID;
    int st = check_params(prm);
    if (st) return fail(ctx, st, "unsupported parameters");
    if (prm->dim != ctx->prm.dim) return fail(ctx, SPH_E_INVALID, "dim cannot change");
    if (ctx->batch) return fail(ctx, SPH_E_STATE, "a batch keeps the parameters it was created with");
    // a precision with mirrors of its own: the walls' mirrors are written once
    // here; so is their pressure tensor, whose form depends on SPH
    const bool to_mixed = (prm->precision != SPH_PREC_FP64 && ctx->prm.precision != prm->precision) ||
                          prm->pa_sph != ctx->prm.pa_sph;
    drop_graph(ctx);
    ctx->prm = *prm;
    fill_common(ctx->d, *prm);
    if (prm->precision != SPH_PREC_FP64 && ensure_mirrors(ctx)) return fail(ctx, SPH_E_NOMEM, "FP32 mirrors");
    if ((st = ensure_options(ctx))) return st;
    ctx->density_done = false;
    HostInst& h = ctx->insts[0];
    h.prm = *prm;
    if (ctx->uploaded) {
        if ((st = pull_instances(ctx))) return st;  // keep the device step counter and time
        h.I.dt = prm->dt;
    }
    if ((st = push_instance(ctx, 0))) return st;
    if (ctx->uploaded) {   // the kernel may have changed: the reference constants with it
        sph::launch_kref(ctx->d, 0, ctx->d.n_real > 0 ? 0 : -1, ctx->stream);
        ++ctx->launches;
        CK(cudaGetLastError());
    }
    if (to_mixed && ctx->uploaded) {
        // wall mirrors are written once; real particles' at the next reorder
        sph::launch_wall_init(ctx->d, ctx->d.wall_off, ctx->d.n_wall, ctx->stream);
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
    if (ctx->batch) return fail(ctx, SPH_E_STATE, "use sph_batch_add on a batch");
    if (n_real < 0 || n_wall < 0 || n_real + n_wall <= 0 || n_real + n_wall > ctx->capacity)
        return fail(ctx, SPH_E_INVALID, "particle count out of range");
    if (!x || !v || !mass || !rho || !p || !e || !c || !h || !type)
        return fail(ctx, SPH_E_INVALID, "null input array");
    drop_graph(ctx);
    Dev& d = ctx->d;
    // a plain context keeps its walls right after its real particles
    d.n_real = 0;
    d.n_wall = 0;
    d.total_cells = 0;
    d.wall_off = (int)n_real;
    ctx->wall_end = n_real;
    ctx->pending_remove = 0;
    int st = add_instance(ctx, 0, ctx->prm, n_real, n_wall, x, v, mass, rho, p, e, c, h, type, state, boundary,
                          shear);
    if (st) return st;
    ctx->step = 0;
    ctx->time = 0.0;
    return SPH_OK;
}

int sph_upload_blocks(sph_ctx* ctx, int32_t n_blocks, const sph_block* blocks, int32_t n_real_blocks) {
    if (!ctx) return SPH_E_INVALID;
    if (ctx->batch) return fail(ctx, SPH_E_STATE, "use sph_batch_add_blocks on a batch");
    int64_t n_real = 0, n_wall = 0;
    int st = check_blocks(ctx, ctx->prm.dim, n_blocks, blocks, n_real_blocks, &n_real, &n_wall);
    if (st) return st;
    if (n_real + n_wall > ctx->capacity) return fail(ctx, SPH_E_INVALID, "particle count out of range");
    drop_graph(ctx);
    Dev& d = ctx->d;
    d.n_real = 0;
    d.n_wall = 0;
    d.total_cells = 0;
    d.wall_off = (int)n_real;
    ctx->wall_end = n_real;
    ctx->pending_remove = 0;
    BlockSource src;
    src.blocks = blocks;
    src.n = n_blocks;
    src.n_real = n_real_blocks;
    st = add_instance(ctx, 0, ctx->prm, n_real, n_wall, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, src);
    if (st) return st;
    ctx->step = 0;
    ctx->time = 0.0;
    return SPH_OK;
}

int sph_download(sph_ctx* ctx, double* x, double* v, double* rho, double* p, double* e, double* c,
                 double* shear) {
    int st = need_plain(ctx, false);
    if (st) return st;
    const int64_t N = ctx->d.n_real + ctx->d.n_wall, dim = ctx->d.dim;
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
    int st = need_plain(ctx, false);
    if (st) return st;
    if (!out || field < SPH_FIELD_X || field > SPH_FIELD_AVER) return fail(ctx, SPH_E_INVALID, "bad field");
    return gather_to_host(ctx, field, out, (int64_t)(ctx->d.n_real + ctx->d.n_wall) * comps_of(ctx->d, field));
}

int sph_set_field(sph_ctx* ctx, int32_t field, const double* in) {
    int st = need_plain(ctx, false);
    if (st) return st;
    if (!in) return fail(ctx, SPH_E_INVALID, "null input");
    const int64_t n = ctx->d.n_real + ctx->d.n_wall;
    const int64_t count = n * comps_of(ctx->d, field);
    CK(cudaMemcpyAsync(ctx->stage, in, sizeof(double) * count, cudaMemcpyHostToDevice, ctx->stream));
    sph::launch_set_field(ctx->d, field, ctx->stage, (int)n, -1, ctx->stream);
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
    if (ctx->batch) return fail(ctx, SPH_E_UNSUPPORTED, "neighbour export of a batch");
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
    int st = need_plain(ctx, true);
    if (st) return st;
    if ((st = kgc_stage(ctx))) return st;
    if ((st = density_stage(ctx))) return st;
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

int sph_arti_heat(sph_ctx* ctx, double* dedt) {
    if (ctx && (ctx->d.precision != SPH_PREC_FP64 || ctx->d.pa_sph != 2 || ctx->d.kgc))
        return fail(ctx, SPH_E_UNSUPPORTED, "artificial heat: FP64, SPH = 2, no kernel correction");
    int st = module_call(ctx, SPH_TERM_ARTI_HEAT, false);
    if (st) return st;
    return gather_to_host(ctx, SPH_FIELD_DEDT, dedt, ctx->d.n_real);
}

int sph_rates(sph_ctx* ctx, double* dvdt, double* drhodt, double* dedt) {
    int st = need_plain(ctx, true);
    if (st) return st;
    if ((st = kgc_stage(ctx))) return st;
    if ((st = density_stage(ctx))) return st;
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
    if ((st = advance_steps(ctx, nsteps))) return st;
    if ((st = check_status_word(ctx))) return st;
    if (max_courant || mean_courant) {
        double cr[3];
        CK(cudaMemcpyAsync(cr, ctx->d.cres, sizeof(cr), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (max_courant) *max_courant = cr[0];
        if (mean_courant) *mean_courant = cr[1];
    }
    return SPH_OK;
}

int sph_advance_async(sph_ctx* ctx, int64_t nsteps) {
    int st = need(ctx, false);
    if (st) return st;
    if (nsteps < 0) return fail(ctx, SPH_E_INVALID, "nsteps < 0");
    return advance_steps(ctx, nsteps);
}

int sph_sync(sph_ctx* ctx, double* max_courant, double* mean_courant) {
    if (!ctx) return SPH_E_INVALID;
    int st = check_status_word(ctx);
    if (st) return st;
    if (max_courant || mean_courant) {
        double cr[3];
        CK(cudaMemcpyAsync(cr, ctx->d.cres, sizeof(cr), cudaMemcpyDeviceToHost, ctx->stream));
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
    if (ctx->batch) return fail(ctx, SPH_E_UNSUPPORTED, "sph_step_host on a batch");
    if (nsteps < 0 || !x || !v || !rho || !e) return fail(ctx, SPH_E_INVALID, "null host array");
    Dev& d = ctx->d;
    const int64_t nr = d.n_real, dim = d.dim;
    cudaStream_t s = ctx->stream;
    double* X = ctx->stage;
    double* V = X + nr * dim;
    double* R = V + nr * dim;
    double* E = R + nr;
    CK(cudaMemcpyAsync(X, x, sizeof(double) * nr * dim, cudaMemcpyHostToDevice, s));
    // With a step to take (and no stress to upload, which reuses the stage),
    // v, rho and e follow x over the host link on a second stream while the
    // first step sorts the cell keys of the new positions; its build_hash
    // waits for them before the reorder.  The state written is the same.
    const bool overlap = nsteps > 0 && nr > 0 && !(shear && d.has_solid);
    if (overlap) {
        if (!ctx->in_stream) {
            CK(cudaStreamCreateWithFlags(&ctx->in_stream, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&ctx->ev_x, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming));
        }
        CK(cudaEventRecord(ctx->ev_x, s));
        CK(cudaStreamWaitEvent(ctx->in_stream, ctx->ev_x, 0));
        CK(cudaMemcpyAsync(V, v, sizeof(double) * nr * dim, cudaMemcpyHostToDevice, ctx->in_stream));
        CK(cudaMemcpyAsync(R, rho, sizeof(double) * nr, cudaMemcpyHostToDevice, ctx->in_stream));
        CK(cudaMemcpyAsync(E, e, sizeof(double) * nr, cudaMemcpyHostToDevice, ctx->in_stream));
        CK(cudaEventRecord(ctx->ev_in, ctx->in_stream));
        sph::launch_host_state(d, 2, ctx->stage, s);
        ctx->rest_pending = true;
    } else {
        CK(cudaMemcpyAsync(V, v, sizeof(double) * nr * dim, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(R, rho, sizeof(double) * nr, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(E, e, sizeof(double) * nr, cudaMemcpyHostToDevice, s));
        sph::launch_host_state(d, 1, ctx->stage, s);
    }
    ++ctx->launches;
    if (shear && d.has_solid) {
        CK(cudaStreamSynchronize(s));
        CK(cudaMemcpyAsync(ctx->stage, shear, sizeof(double) * nr * d.d2, cudaMemcpyHostToDevice, s));
        sph::launch_set_field(d, SPH_FIELD_SHEAR, ctx->stage, (int)nr, -1, s);
        ++ctx->launches;
    }
    CK(cudaGetLastError());
    ctx->hash_valid = false;
    for (int64_t k = 0; k < nsteps; ++k) {
        if ((st = one_step(ctx))) {
            if (ctx->rest_pending) {   // no reorder ran: leave no copy in flight
                ctx->rest_pending = false;
                cudaStreamSynchronize(ctx->in_stream);
            }
            return st;
        }
    }
    sph::launch_host_state(d, 0, ctx->stage, s);
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

int sph_boundary(sph_ctx* ctx, double* dvdt) {
    int st = need_plain(ctx, false);
    if (st) return st;
    const int64_t n = (int64_t)ctx->d.n_real * ctx->d.dim;
    if (dvdt) CK(cudaMemcpyAsync(ctx->stage, dvdt, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    sph::launch_boundary(ctx->d, dvdt ? ctx->stage : nullptr, ctx->stream);
    ++ctx->launches;
    CK(cudaGetLastError());
    if (dvdt) CK(cudaMemcpyAsync(dvdt, ctx->stage, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_courant_num(sph_ctx* ctx, int64_t n, const double* hsml, const double* div_v, const double* c,
                    double* xi) {
    if (!ctx) return SPH_E_INVALID;
    if (n < 0 || (n > 0 && (!hsml || !div_v || !c || !xi))) return fail(ctx, SPH_E_INVALID, "courant_num arrays");
    if (ctx->batch) return fail(ctx, SPH_E_UNSUPPORTED, "courant_num of a batch: its systems have their own dt");
    // chunks of three arrays through the staging buffer; xi overwrites h
    const int64_t chunk = std::min<int64_t>(ctx->stage_bytes / (3 * sizeof(double)), 1 << 30);
    double* H = ctx->stage;
    double* DV = H + chunk;
    double* C = DV + chunk;
    const sph_params& p = ctx->insts[0].prm;
    for (int64_t o = 0; o < n; o += chunk) {
        const int64_t m = std::min(chunk, n - o);
        CK(cudaMemcpyAsync(H, hsml + o, sizeof(double) * m, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(DV, div_v + o, sizeof(double) * m, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(C, c + o, sizeof(double) * m, cudaMemcpyHostToDevice, ctx->stream));
        sph::launch_courant_num((int)m, p.dt, p.cour_alpha, p.cour_beta, H, DV, C, H, ctx->stream);
        ++ctx->launches;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(xi + o, H, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return SPH_OK;
}

int sph_energy(sph_ctx* ctx, int32_t inst, double out[4]) {
    if (!out) return fail(ctx, SPH_E_INVALID, "null output");
    int st = need(ctx, false);
    if (st) return st;
    if (inst >= 0 && (st = inst_index(ctx, inst))) return st;
    if (!ctx->batch) inst = -1;
    // the staging buffer holds the block partials (3 per 256 particles) and
    // the three sums after them
    double* part = ctx->stage;
    const int64_t nb = (ctx->d.n_real + 255) / 256;
    double* sums = part + 3 * nb;
    ctx->launches += sph::launch_energy(ctx->d, inst, part, sums, ctx->stream);
    CK(cudaGetLastError());
    double h[3];
    CK(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out[0] = h[0]; out[1] = h[1]; out[2] = h[2];
    out[3] = (h[0] + h[1]) + h[2];
    return SPH_OK;
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

// ---- batches ----------------------------------------------------------------

int sph_batch_create(const sph_params* prm, int32_t max_instances, int64_t real_capacity,
                     int64_t wall_capacity, sph_ctx** out) {
    if (!out) return SPH_E_INVALID;
    *out = nullptr;
    int st = check_params(prm);
    if (st) return st;
    if (max_instances <= 0 || real_capacity <= 0 || wall_capacity < 0 ||
        real_capacity + wall_capacity >= ((int64_t)1 << 31))
        return SPH_E_INVALID;
    st = create_ctx(prm, max_instances, real_capacity + wall_capacity, out);
    if (st) return st;
    sph_ctx* ctx = *out;
    ctx->batch = true;
    ctx->real_cap = real_capacity;
    ctx->d.wall_off = (int)real_capacity;
    ctx->wall_end = real_capacity;
    return SPH_OK;
}

int sph_batch_add(sph_ctx* ctx, const sph_params* prm, int64_t n_real, int64_t n_wall, const double* x,
                  const double* v, const double* mass, const double* rho, const double* p, const double* e,
                  const double* c, const double* h, const int32_t* type, const int32_t* state,
                  const int32_t* boundary, const double* shear, int32_t* inst) {
    if (!ctx || !inst) return SPH_E_INVALID;
    if (!ctx->batch) return fail(ctx, SPH_E_STATE, "not a batch context");
    int st = check_params(prm);
    if (st) return fail(ctx, st, "unsupported parameters");
    if (!same_model(*prm, ctx->prm)) return fail(ctx, SPH_E_INVALID, "instance model differs from the batch");
    if (n_real <= 0 || n_wall < 0 || !x || !v || !mass || !rho || !p || !e || !c || !h || !type)
        return fail(ctx, SPH_E_INVALID, "bad instance arrays");
    if (state)
        for (int64_t q = n_real; q < n_real + n_wall; ++q)
            if (state[q] == -1) return fail(ctx, SPH_E_UNSUPPORTED, "State = -1 wall particles in a batch");
    if (ctx->d.n_real - ctx->pending_remove + n_real > ctx->real_cap)
        return fail(ctx, SPH_E_NOMEM, "real-particle capacity of the batch exhausted");
    if (ctx->wall_end + n_wall > ctx->capacity) return fail(ctx, SPH_E_NOMEM, "wall capacity of the batch exhausted");
    int k = -1;
    for (int q = 0; q < ctx->max_inst; ++q)
        if (!ctx->insts[q].used) { k = q; break; }
    if (k < 0) return fail(ctx, SPH_E_NOMEM, "no free instance slot");
    if (ctx->pending_remove) {  // drop removed particles before appending
        if ((st = build_hash(ctx, false))) return st;
        CK(cudaStreamSynchronize(ctx->stream));
    }
    drop_graph(ctx);
    st = add_instance(ctx, k, *prm, n_real, n_wall, x, v, mass, rho, p, e, c, h, type, state, boundary, shear);
    if (st) {
        ctx->insts[k].used = false;
        return st;
    }
    *inst = k;
    return SPH_OK;
}

int sph_batch_add_blocks(sph_ctx* ctx, const sph_params* prm, int32_t n_blocks, const sph_block* blocks,
                         int32_t n_real_blocks, int32_t* inst) {
    if (!ctx || !inst) return SPH_E_INVALID;
    if (!ctx->batch) return fail(ctx, SPH_E_STATE, "not a batch context");
    int st = check_params(prm);
    if (st) return fail(ctx, st, "unsupported parameters");
    if (!same_model(*prm, ctx->prm)) return fail(ctx, SPH_E_INVALID, "instance model differs from the batch");
    int64_t n_real = 0, n_wall = 0;
    if ((st = check_blocks(ctx, ctx->prm.dim, n_blocks, blocks, n_real_blocks, &n_real, &n_wall))) return st;
    for (int b = 0; b < n_blocks; ++b)
        if (b >= n_real_blocks && blocks[b].state == -1)
            return fail(ctx, SPH_E_UNSUPPORTED, "State = -1 wall particles in a batch");
    if (ctx->d.n_real - ctx->pending_remove + n_real > ctx->real_cap)
        return fail(ctx, SPH_E_NOMEM, "real-particle capacity of the batch exhausted");
    if (ctx->wall_end + n_wall > ctx->capacity) return fail(ctx, SPH_E_NOMEM, "wall capacity of the batch exhausted");
    int k = -1;
    for (int q = 0; q < ctx->max_inst; ++q)
        if (!ctx->insts[q].used) { k = q; break; }
    if (k < 0) return fail(ctx, SPH_E_NOMEM, "no free instance slot");
    if (ctx->pending_remove) {  // drop removed particles before appending
        if ((st = build_hash(ctx, false))) return st;
        CK(cudaStreamSynchronize(ctx->stream));
    }
    drop_graph(ctx);
    BlockSource src;
    src.blocks = blocks;
    src.n = n_blocks;
    src.n_real = n_real_blocks;
    st = add_instance(ctx, k, *prm, n_real, n_wall, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, nullptr, nullptr, nullptr, nullptr, src);
    if (st) {
        ctx->insts[k].used = false;
        return st;
    }
    *inst = k;
    return SPH_OK;
}

int sph_batch_remove(sph_ctx* ctx, int32_t inst) {
    int st = inst_index(ctx, inst);
    if (st) return st;
    HostInst& h = ctx->insts[inst];
    drop_graph(ctx);
    if ((st = pull_instances(ctx))) return st;
    h.I.active = 0;
    if ((st = push_instance(ctx, inst))) return st;
    // its real particles sort to the end at the next reorder and are dropped;
    // its walls and cells stay until the slot is reused or the batch compacts
    ctx->pending_remove += h.n_real;
    h.used = false;
    ctx->hash_valid = false;
    return SPH_OK;
}

int sph_batch_get_field(sph_ctx* ctx, int32_t inst, int32_t field, double* out) {
    int st = inst_index(ctx, inst);
    if (st) return st;
    if (!out || field < SPH_FIELD_X || field > SPH_FIELD_AVER) return fail(ctx, SPH_E_INVALID, "bad field");
    const HostInst& h = ctx->insts[inst];
    return gather_to_host(ctx, field, out, (h.n_real + h.n_wall) * comps_of(ctx->d, field), inst);
}

int sph_batch_info(sph_ctx* ctx, int32_t inst, int64_t* n_real, int64_t* n_wall, int64_t* step, double* time,
                   double* max_courant, double* mean_courant) {
    int st = inst_index(ctx, inst);
    if (st) return st;
    if ((st = pull_instances(ctx))) return st;
    const HostInst& h = ctx->insts[inst];
    if (n_real) *n_real = h.n_real;
    if (n_wall) *n_wall = h.n_wall;
    if (step) *step = h.I.step;
    if (time) *time = h.I.time;
    if (max_courant || mean_courant) {
        double cr[3];
        CK(cudaMemcpyAsync(cr, ctx->d.cres + 3 * inst, sizeof(cr), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (max_courant) *max_courant = cr[0];
        if (mean_courant) *mean_courant = cr[1];
    }
    return SPH_OK;
}

int sph_batch_capacity(sph_ctx* ctx, int64_t* free_real, int64_t* free_wall, int32_t* free_slots) {
    if (!ctx || !ctx->batch) return SPH_E_INVALID;
    if (free_real) *free_real = ctx->real_cap - (ctx->d.n_real - ctx->pending_remove);
    if (free_wall) *free_wall = ctx->capacity - ctx->wall_end;
    if (free_slots) {
        int f = 0;
        for (auto& h : ctx->insts) f += h.used ? 0 : 1;
        *free_slots = f;
    }
    return SPH_OK;
}

int sph_batch_slots(sph_ctx* ctx, int32_t* max_instances, uint8_t* live) {
    if (!ctx || !max_instances) return SPH_E_INVALID;
    if (!ctx->batch) return fail(ctx, SPH_E_STATE, "not a batch context");
    *max_instances = ctx->max_inst;
    if (live)
        for (int k = 0; k < ctx->max_inst; ++k)
            live[k] = ctx->insts[k].used && ctx->insts[k].I.active ? 1 : 0;
    return SPH_OK;
}

// ---- status, streams, timing ------------------------------------------------

int sph_status(sph_ctx* ctx, char* msg, size_t len) {
    if (!ctx) return SPH_E_INVALID;
    if (msg && len) std::snprintf(msg, len, "%s", ctx->msg.c_str());
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

int sph_set_option(sph_ctx* ctx, int32_t option, double value) {
    if (!ctx) return SPH_E_INVALID;
    switch (option) {
    case SPH_OPT_GRAPHS:
        ctx->use_graphs = value != 0.0;
        if (!ctx->use_graphs) drop_graph(ctx);
        return SPH_OK;
    case SPH_OPT_SMEM_CARVEOUT:
        sph::set_pass_carveout((int)value);
        drop_graph(ctx);
        return SPH_OK;
    case SPH_OPT_BLOCK_SIZE:
    case SPH_OPT_LIST_LEN: {
        const int v = (int)value;
        int tpb = ctx->d.tile_tpb, k = ctx->d.tile_k;
        if (option == SPH_OPT_BLOCK_SIZE) {
            if (v != 32 && v != 64 && v != 128) return fail(ctx, SPH_E_INVALID, "block size: 32, 64 or 128");
            tpb = v;
        } else {
            if (v != 64 && v != 88 && v != 120) return fail(ctx, SPH_E_INVALID, "list length: 64, 88 or 120");
            k = v;
        }
        const size_t smem = sph::tiled_smem_bytes(tpb, k);
        if (smem > 227 * 1024) return fail(ctx, SPH_E_INVALID, "block size x list length needs more than 227 KB");
        if (smem > 48 * 1024 && sph::set_tiled_smem_limit(smem) != 0)
            return fail(ctx, SPH_E_CUDA, "cannot raise the dynamic shared memory limit");
        ctx->d.tile_tpb = tpb;
        ctx->d.tile_k = k;
        drop_graph(ctx);
        return SPH_OK;
    }
    case SPH_OPT_PERSISTENT:
        if (value != 0.0 && value != 1.0) return fail(ctx, SPH_E_INVALID, "persistent: 0 or 1");
        ctx->d.persistent = value != 0.0 ? 1 : 0;
        drop_graph(ctx);
        return SPH_OK;
    case SPH_OPT_LANES: {
        int sh = -1;
        for (int k = 0; k <= 5; ++k)
            if (value == (double)(1 << k)) sh = k;
        if (sh < 0) return fail(ctx, SPH_E_INVALID, "lanes: 1, 2, 4, 8, 16 or 32");
        ctx->d.lane_shift = sh;
        drop_graph(ctx);
        return SPH_OK;
    }
    default:
        return fail(ctx, SPH_E_INVALID, "unknown option");
    }
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

int sph_get_params(sph_ctx* ctx, sph_params* out) {
    if (!ctx || !out) return SPH_E_INVALID;
    *out = ctx->prm;
    return SPH_OK;
}

int sph_check_conversions(int64_t n, uint64_t seed, int64_t* mismatches) {
    if (!mismatches || n < 0) return SPH_E_INVALID;
    unsigned long long* bad = nullptr;
    if (cudaMalloc((void**)&bad, sizeof(*bad)) != cudaSuccess) { cudaGetLastError(); return SPH_E_NOMEM; }
    unsigned long long h = 0;
    cudaError_t e = cudaMemset(bad, 0, sizeof(*bad));
    if (e == cudaSuccess) {
        sph::launch_conversion_check(n, seed, bad, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    if (e != cudaSuccess) return SPH_E_CUDA;
    *mismatches = (int64_t)h;
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

int sph_state_bytes(sph_ctx* ctx, int64_t* bytes) {
    if (!ctx || !bytes) return SPH_E_INVALID;
    if (!ctx->uploaded) return fail(ctx, SPH_E_STATE, "no particles uploaded");
    *bytes = (int64_t)sizeof(StateHeader) + state_payload(ctx);
    return SPH_OK;
}

int sph_state_save(sph_ctx* ctx, void* buffer, int64_t size) {
    if (!ctx || !buffer) return SPH_E_INVALID;
    if (!ctx->uploaded) return fail(ctx, SPH_E_STATE, "no particles uploaded");
    const int64_t payload = state_payload(ctx);
    if (size < (int64_t)sizeof(StateHeader) + payload) return fail(ctx, SPH_E_INVALID, "buffer too small");
    int st = pull_instances(ctx);  // device-updated step counters and times
    if (st) return st;
    StateHeader h{};
    std::memcpy(h.magic, kStateMagic, sizeof(h.magic));
    h.version = kStateVersion;
    h.header_bytes = sizeof(StateHeader);
    h.params_bytes = sizeof(sph_params);
    h.inst_bytes = sizeof(sph::Inst);
    h.material_bytes = sizeof(sph::DevMaterial);
    h.prm = ctx->prm;
    h.batch = ctx->batch;
    h.max_inst = ctx->max_inst;
    h.has_solid = ctx->d.has_solid;
    h.mirrors = ctx->d.pr4 != nullptr;
    h.dxp = ctx->d.dxp != nullptr;
    h.key_bits = ctx->key_bits;
    h.capacity = ctx->capacity;
    h.real_cap = ctx->real_cap;
    h.wall_end = ctx->wall_end;
    h.cell_cap = ctx->cell_cap;
    h.pending_remove = ctx->pending_remove;
    h.n_real = ctx->d.n_real;
    h.n_wall = ctx->d.n_wall;
    h.wall_off = ctx->d.wall_off;
    h.total_cells = ctx->d.total_cells;
    h.step = ctx->step;
    h.time = ctx->time;
    h.payload_bytes = payload;
    unsigned char* out = (unsigned char*)buffer;
    std::memcpy(out, &h, sizeof(h));
    out += sizeof(h);
    for (int k = 0; k < ctx->max_inst; ++k) {
        const HostInst& hi = ctx->insts[k];
        StateInst si{};
        si.I = hi.I;
        si.prm = hi.prm;
        si.n_real = hi.n_real;
        si.n_wall = hi.n_wall;
        si.wall_first = hi.wall_first;
        si.used = hi.used;
        std::memcpy(out, &si, sizeof(si));
        out += sizeof(si);
    }
    return state_copy(ctx, out, true);
}

// A checkpoint's instance record may only point inside the checkpoint's own
// ranges: its real particles within n_real, its walls within the wall slots,
// its cells within total_cells and its material rows within its own block
// of the material table.  A corrupted or hand-edited buffer fails here
// instead of driving the kernels out of range.
static bool state_inst_ok(const StateHeader& h, const StateInst& si, int k) {
    if (!si.used) return true;
    const sph::Inst& I = si.I;
    if (si.n_real < 0 || si.n_real > h.n_real || si.n_wall < 0 || si.wall_first < 0) return false;
    if (si.n_wall > 0 && (si.wall_first < h.wall_off || si.wall_first + si.n_wall > h.wall_end)) return false;
    if (I.n_real < 0 || I.n_real > h.n_real || I.n_wall != si.n_wall || I.wall_first != si.wall_first) return false;
    const int dim = h.prm.dim;
    int64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        if (I.grid.nc[a] < 1 || (a >= dim && I.grid.nc[a] != 1)) return false;
        cells *= I.grid.nc[a];
    }
    if (cells != I.grid.ncells || !(I.grid.cs > 0.0) || !(I.grid.inv_cs > 0.0) || !std::isfinite(I.grid.cs))
        return false;
    if (I.cell_base < 0 || (int64_t)I.cell_base + I.grid.ncells > h.total_cells) return false;
    if (h.total_cells > (int64_t)INT32_MAX - 2) return false;   // keys below 2^31
    unsigned long long m[2];
    int l[2];
    grid_divisors(I.grid, m, l);   // the cell of a key is decoded with them
    if (m[0] != I.grid.div_m[0] || m[1] != I.grid.div_m[1] || l[0] != I.grid.div_l[0] || l[1] != I.grid.div_l[1])
        return false;
    if (I.mat_base != k * SPH_MAX_MATERIALS || I.n_mat < 0 || I.n_mat > SPH_MAX_MATERIALS) return false;
    return si.prm.dim == dim;
}

int sph_state_load(const void* buffer, int64_t size, sph_ctx** out) {
    if (!buffer || !out) return SPH_E_INVALID;
    *out = nullptr;
    StateHeader h;
    if (size < (int64_t)sizeof(h)) return SPH_E_INVALID;
    std::memcpy(&h, buffer, sizeof(h));
    if (std::memcmp(h.magic, kStateMagic, sizeof(h.magic)) != 0 || h.version != kStateVersion ||
        h.header_bytes != sizeof(StateHeader) || h.params_bytes != sizeof(sph_params) ||
        h.inst_bytes != sizeof(sph::Inst) || h.material_bytes != sizeof(sph::DevMaterial))
        return SPH_E_INVALID;
    if (size < (int64_t)sizeof(h) + h.payload_bytes) return SPH_E_INVALID;
    if (h.max_inst <= 0 || h.capacity <= 0 || h.capacity >= ((int64_t)1 << 31) || h.n_real < 0 ||
        h.wall_off < h.n_real || h.wall_end < h.wall_off || h.wall_end > h.capacity || h.cell_cap < 0 ||
        h.total_cells < 0 || h.total_cells > h.cell_cap || h.n_wall < 0 || h.max_inst > (1 << 20) ||
        h.key_bits < 1 || h.key_bits > 32 || ((int64_t)1 << h.key_bits) <= h.total_cells + 1 ||
        (h.batch && (h.real_cap < h.n_real || h.real_cap > h.wall_off)))
        return SPH_E_INVALID;
    {
        // instance records sit right after the header (bounded by the payload
        // size checked above); look at them before allocating anything
        const unsigned char* rec = (const unsigned char*)buffer + sizeof(h);
        if (h.payload_bytes < (int64_t)sizeof(StateInst) * h.max_inst) return SPH_E_INVALID;
        for (int k = 0; k < h.max_inst; ++k) {
            StateInst si;
            std::memcpy(&si, rec + (size_t)k * sizeof(si), sizeof(si));
            if (!state_inst_ok(h, si, k)) return SPH_E_INVALID;
        }
    }
    int st = check_params(&h.prm);
    if (st) return st;
    sph_ctx* ctx = nullptr;
    if ((st = create_ctx(&h.prm, h.max_inst, h.capacity, &ctx))) return st;
    auto bail = [&](int code) { sph_destroy(ctx); return code; };
    ctx->batch = h.batch != 0;
    ctx->real_cap = h.real_cap;
    if (h.has_solid && ensure_solid(ctx)) return bail(SPH_E_NOMEM);
    if (h.mirrors && ensure_mirrors(ctx)) return bail(SPH_E_NOMEM);
    if (h.dxp != (ctx->d.dxp != nullptr)) return bail(SPH_E_INVALID);
    if (h.cell_cap > 0 && ensure_cells(ctx, h.cell_cap)) return bail(SPH_E_NOMEM);
    if (ctx->cell_cap != h.cell_cap) return bail(SPH_E_INVALID);
    Dev& d = ctx->d;
    d.n_real = (int)h.n_real;
    d.n_wall = (int)h.n_wall;
    d.wall_off = (int)h.wall_off;
    d.total_cells = (int)h.total_cells;
    ctx->wall_end = h.wall_end;
    ctx->pending_remove = h.pending_remove;
    ctx->key_bits = h.key_bits;
    ctx->step = h.step;
    ctx->time = h.time;
    if (state_payload(ctx) != h.payload_bytes) return bail(SPH_E_INVALID);
    const unsigned char* in = (const unsigned char*)buffer + sizeof(h);
    for (int k = 0; k < h.max_inst; ++k) {
        StateInst si;
        std::memcpy(&si, in, sizeof(si));
        in += sizeof(si);
        HostInst& hi = ctx->insts[k];
        hi.I = si.I;
        hi.prm = si.prm;
        hi.n_real = si.n_real;
        hi.n_wall = si.n_wall;
        hi.wall_first = si.wall_first;
        hi.used = si.used != 0;
    }
    if ((st = state_copy(ctx, const_cast<unsigned char*>(in), false))) return bail(st);
    ctx->uploaded = true;
    ctx->hash_valid = false;
    ctx->density_done = false;
    *out = ctx;
    return SPH_OK;
}

}  // extern "C"
