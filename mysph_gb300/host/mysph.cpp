// mysph.cpp — the module procedures of mysph.hpp on libsphgpu.
#include "mysph.hpp"

#include <algorithm>
#include <cstring>
#include <sstream>

namespace mysph {

Error::Error(int st, const std::string& where, const std::string& msg)
    : std::runtime_error(where + " failed with status " + std::to_string(st) + (msg.empty() ? "" : ": " + msg)),
      status(st) {}

void Field::check(int st, const char* where) const {
    if (st == SPH_OK) return;
    char msg[512] = {0};
    if (ctx) sph_status(ctx, msg, sizeof(msg));
    throw Error(st, where, msg);
}

Field::Field(const sph_params& prm, std::vector<Particle>& parts, int nt, int nd, const std::vector<double>* shear)
    : Dim(prm.dim), ntotal(nt), ndummy(nd), P(parts) {
    const int N = nt + nd;
    if (N <= 0 || (int)P.size() < N) throw Error(SPH_E_INVALID, "Field", "fewer particles than ntotal + ndummy");
    check(sph_create(&prm, N, &ctx), "sph_create");
    std::vector<double> x(N * Dim), v(N * Dim), m(N), rho(N), p(N), e(N), c(N), h(N);
    std::vector<int32_t> type(N), state(N), bnd(N);
    for (int i = 0; i < N; ++i) {
        const Particle& q = P[i];
        for (int a = 0; a < Dim; ++a) { x[i * Dim + a] = q.x[a]; v[i * Dim + a] = q.v[a]; }
        m[i] = q.Mass; rho[i] = q.Density; p[i] = q.Pressure; e[i] = q.InternalEnergy;
        c[i] = q.SoundSpeed; h[i] = q.SmoothingLength;
        type[i] = q.Type; state[i] = q.State; bnd[i] = q.Boundary;
    }
    const int st = sph_upload(ctx, nt, nd, x.data(), v.data(), m.data(), rho.data(), p.data(), e.data(), c.data(),
                              h.data(), type.data(), state.data(), bnd.data(), shear ? shear->data() : nullptr);
    if (st != SPH_OK) {
        char msg[512] = {0};
        sph_status(ctx, msg, sizeof(msg));
        sph_destroy(ctx);
        ctx = nullptr;
        throw Error(st, "sph_upload", msg);
    }
}

Field::~Field() {
    if (ctx) sph_destroy(ctx);
}

std::vector<double> Field::field(int32_t id) const {
    const int N = ntotal + ndummy, D2 = Dim * Dim;
    const int comps = (id == SPH_FIELD_X || id == SPH_FIELD_V || id == SPH_FIELD_DISP || id == SPH_FIELD_DVDT ||
                       id == SPH_FIELD_AVER) ? Dim
                      : (id == SPH_FIELD_STRESS || id == SPH_FIELD_SHEAR || id == SPH_FIELD_DSDT ||
                         id == SPH_FIELD_STRAIN) ? D2 : 1;
    std::vector<double> out((size_t)N * comps);
    check(sph_get_field(ctx, id, out.data()), "sph_get_field");
    return out;
}

double Field::time() const {
    int64_t nr, nw, st;
    double t;
    check(sph_info(ctx, &nr, &nw, &st, &t), "sph_info");
    return t;
}

long long Field::step() const {
    int64_t nr, nw, st;
    double t;
    check(sph_info(ctx, &nr, &nw, &st, &t), "sph_info");
    return st;
}

void Field::pull() {
    const int N = ntotal + ndummy, D2 = Dim * Dim;
    const auto x = field(SPH_FIELD_X), v = field(SPH_FIELD_V), rho = field(SPH_FIELD_RHO), p = field(SPH_FIELD_P);
    const auto e = field(SPH_FIELD_E), c = field(SPH_FIELD_C), dsp = field(SPH_FIELD_DISP);
    const auto stress = field(SPH_FIELD_STRESS), dx = field(SPH_FIELD_DIVX), dv = field(SPH_FIELD_DIVV);
    for (int i = 0; i < N; ++i) {
        Particle& q = P[i];
        for (int a = 0; a < Dim; ++a) {
            q.x[a] = x[i * Dim + a];
            q.v[a] = v[i * Dim + a];
            q.Displacement[a] = dsp[i * Dim + a];
        }
        for (int k = 0; k < D2; ++k) q.Stress[k] = stress[i * D2 + k];
        q.Density = rho[i]; q.Pressure = p[i]; q.InternalEnergy = e[i]; q.SoundSpeed = c[i];
        q.divergencePosition = dx[i]; q.divergenceVelocity = dv[i];
    }
}

static std::vector<Vec> vecs(const std::vector<double>& a, int n, int dim) {
    std::vector<Vec> out(n, Vec{0, 0, 0});
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < dim; ++d) out[i][d] = a[(size_t)i * dim + d];
    return out;
}

void BGGS(Field& f) {
    f.check(sph_nnps(f.ctx), "sph_nnps");
    int64_t total = 0;
    f.check(sph_neighbor_counts(f.ctx, nullptr, &total), "sph_neighbor_counts");
    std::vector<int64_t> off(f.ntotal + 1);
    std::vector<int32_t> lst(std::max<int64_t>(total, 1));
    f.check(sph_export_neighbors(f.ctx, off.data(), lst.data(), total), "sph_export_neighbors");
    for (int i = 0; i < f.ntotal; ++i) {
        Particle& q = f.P[i];
        q.neighborNum = (int)(off[i + 1] - off[i]);
        q.neighborList.assign(lst.begin() + off[i], lst.begin() + off[i + 1]);
    }
}

void con_density(Field& f, int ntotal, std::vector<double>& drhodt) {
    drhodt.assign(ntotal, 0.0);
    f.check(sph_density(f.ctx, drhodt.data()), "sph_density");
}

void sum_density(Field& f, int ntotal) {
    std::vector<double> unused(ntotal);
    f.check(sph_density(f.ctx, unused.data()), "sph_density");
    const auto rho = f.field(SPH_FIELD_RHO);
    for (int i = 0; i < ntotal; ++i) f.P[i].Density = rho[i];
}

void divergence(Field& f, int ntotal) {
    std::vector<double> dx(ntotal), dv(ntotal);
    f.check(sph_divergence(f.ctx, dx.data(), dv.data()), "sph_divergence");
    for (int i = 0; i < ntotal; ++i) {
        f.P[i].divergencePosition = dx[i];
        f.P[i].divergenceVelocity = dv[i];
    }
}

void internal_force(Field& f, int ntotal, std::vector<Vec>& dvdt, std::vector<double>& dedt) {
    std::vector<double> a((size_t)ntotal * f.Dim);
    dedt.assign(ntotal, 0.0);
    f.check(sph_internal_force(f.ctx, a.data(), dedt.data(), nullptr), "sph_internal_force");
    dvdt = vecs(a, ntotal, f.Dim);
}

void external_force(Field& f, int ntotal, std::vector<Vec>& dvdt) {
    std::vector<double> a((size_t)ntotal * f.Dim);
    f.check(sph_external_force(f.ctx, a.data()), "sph_external_force");
    dvdt = vecs(a, ntotal, f.Dim);
}

void arti_visc(Field& f, int ntotal, std::vector<Vec>& dvdt, std::vector<double>& dedt) {
    std::vector<double> a((size_t)ntotal * f.Dim);
    dedt.assign(ntotal, 0.0);
    f.check(sph_arti_visc(f.ctx, a.data(), dedt.data()), "sph_arti_visc");
    dvdt = vecs(a, ntotal, f.Dim);
}

void artificialStress(Field& f, int ntotal, std::vector<Vec>& dvdt) {
    std::vector<double> a((size_t)ntotal * f.Dim);
    f.check(sph_arti_stress(f.ctx, a.data()), "sph_arti_stress");
    dvdt = vecs(a, ntotal, f.Dim);
}

void arti_heat(Field& f, int ntotal, std::vector<double>& dedt) {
    dedt.assign(ntotal, 0.0);
    f.check(sph_arti_heat(f.ctx, dedt.data()), "sph_arti_heat");
}

void boundary(Field& f, int ntotal, std::vector<Update>& Delta) {
    if ((int)Delta.size() < ntotal) throw Error(SPH_E_INVALID, "boundary", "Delta shorter than ntotal");
    std::vector<double> a((size_t)ntotal * f.Dim);
    for (int i = 0; i < ntotal; ++i)
        for (int d = 0; d < f.Dim; ++d) a[(size_t)i * f.Dim + d] = Delta[i].Velocity[d];
    f.check(sph_boundary(f.ctx, a.data()), "sph_boundary");
    for (int i = 0; i < ntotal; ++i)
        for (int d = 0; d < f.Dim; ++d) Delta[i].Velocity[d] = a[(size_t)i * f.Dim + d];
}

std::vector<double> courant_num(Field& f, const std::vector<double>& hsml, const std::vector<double>& div_v,
                                const std::vector<double>& c) {
    if (hsml.size() != div_v.size() || hsml.size() != c.size())
        throw Error(SPH_E_INVALID, "courant_num", "arrays of different lengths");
    std::vector<double> xi(hsml.size());
    f.check(sph_courant_num(f.ctx, (int64_t)hsml.size(), hsml.data(), div_v.data(), c.data(), xi.data()),
            "sph_courant_num");
    return xi;
}

void single_step(Field& f, int ntotal, std::vector<Update>& Delta) {
    std::vector<double> a((size_t)ntotal * f.Dim), drho(ntotal), de(ntotal);
    f.check(sph_rates(f.ctx, a.data(), drho.data(), de.data()), "sph_rates");
    Delta.assign(ntotal, Update{});
    for (int i = 0; i < ntotal; ++i) {
        for (int d = 0; d < f.Dim; ++d) Delta[i].Velocity[d] = a[(size_t)i * f.Dim + d];
        Delta[i].Density = drho[i];
        Delta[i].Energy = de[i];
    }
}

void time_integration(Field& f, long long nsteps, double& max_courant, double& aver_courant) {
    f.check(sph_advance(f.ctx, nsteps, &max_courant, &aver_courant), "sph_advance");
    f.pull();
}

void print_statistics(Field& f, std::ostream& out) {
    double s[6];
    f.check(sph_statistics(f.ctx, s), "sph_statistics");
    out << " >> Statistics: max neighbours " << (long long)s[0] << " (particle " << (long long)s[4]
        << "), min " << (long long)s[1] << " (particle " << (long long)s[5] << "), average " << s[2]
        << ", without neighbours " << (long long)s[3] << "\n";
}

}  // namespace mysph
