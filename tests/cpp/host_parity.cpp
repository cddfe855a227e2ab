// A C++ host of libsphgpu written against mysph.hpp, the way a compiled
// mySPH driver calls its modules: it reads a particle system, runs BGGS and
// the module procedures on it, one single_step and time_integration, and
// writes every result for comparison with the oracle.
//
//   host_parity <case.bin> <out.bin> <nsteps>
//
// case.bin: int32 dim, ntotal, ndummy, params_bytes; sph_params; then
// x, v (N*dim f64), mass, rho, p, e, c, h (N f64), type, state, boundary
// (N int32).  out.bin: int64 neighbour total; int32 neighborNum[ntotal];
// f64 drhodt, divx, divv [ntotal], internal dvdt [ntotal*dim], Delta
// velocity [ntotal*dim], density, energy [ntotal]; then after nsteps:
// x, v [ntotal*dim], rho [ntotal], max and mean Courant.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <vector>

#include "../../mysph_gb300/host/mysph.hpp"

template <class T>
static bool rd(FILE* f, T* p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <class T>
static void wr(FILE* f, const T* p, size_t n) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char** argv) {
    if (argc != 4) { std::cerr << "usage: host_parity case.bin out.bin nsteps\n"; return 2; }
    FILE* in = fopen(argv[1], "rb");
    if (!in) { std::cerr << "cannot read " << argv[1] << "\n"; return 2; }
    int32_t hdr[4];
    sph_params prm;
    if (!rd(in, hdr, 4) || hdr[3] != (int32_t)sizeof(sph_params) || !rd(in, &prm, 1)) {
        std::cerr << "bad header\n";
        return 2;
    }
    const int dim = hdr[0], ntotal = hdr[1], ndummy = hdr[2], N = ntotal + ndummy;
    std::vector<double> x(N * dim), v(N * dim), col[6];
    std::vector<int32_t> it[3];
    bool ok = rd(in, x.data(), x.size()) && rd(in, v.data(), v.size());
    for (auto& c : col) { c.resize(N); ok = ok && rd(in, c.data(), N); }
    for (auto& c : it) { c.resize(N); ok = ok && rd(in, c.data(), N); }
    fclose(in);
    if (!ok) { std::cerr << "short case file\n"; return 2; }

    std::vector<mysph::Particle> P(N);
    for (int i = 0; i < N; ++i) {
        for (int a = 0; a < dim; ++a) { P[i].x[a] = x[i * dim + a]; P[i].v[a] = v[i * dim + a]; }
        P[i].Mass = col[0][i]; P[i].Density = col[1][i]; P[i].Pressure = col[2][i];
        P[i].InternalEnergy = col[3][i]; P[i].SoundSpeed = col[4][i]; P[i].SmoothingLength = col[5][i];
        P[i].Type = it[0][i]; P[i].State = it[1][i]; P[i].Boundary = it[2][i];
    }
    try {
        mysph::Field field(prm, P, ntotal, ndummy);
        mysph::BGGS(field);
        int64_t total = 0;
        std::vector<int32_t> nn(ntotal);
        for (int i = 0; i < ntotal; ++i) { nn[i] = P[i].neighborNum; total += P[i].neighborNum; }
        std::vector<double> drhodt, dedt;
        mysph::con_density(field, ntotal, drhodt);
        mysph::divergence(field, ntotal);
        std::vector<double> divx(ntotal), divv(ntotal);  // time_integration refreshes P
        for (int i = 0; i < ntotal; ++i) { divx[i] = P[i].divergencePosition; divv[i] = P[i].divergenceVelocity; }
        std::vector<mysph::Vec> a_in;
        mysph::internal_force(field, ntotal, a_in, dedt);
        std::vector<mysph::Update> Delta;
        mysph::single_step(field, ntotal, Delta);
        mysph::print_statistics(field, std::cout);
        double mx = 0, mean = 0;
        mysph::time_integration(field, std::atoll(argv[3]), mx, mean);

        FILE* out = fopen(argv[2], "wb");
        if (!out) { std::cerr << "cannot write " << argv[2] << "\n"; return 2; }
        wr(out, &total, 1);
        wr(out, nn.data(), nn.size());
        std::vector<double> buf(ntotal);
        wr(out, drhodt.data(), ntotal);
        wr(out, divx.data(), ntotal);
        wr(out, divv.data(), ntotal);
        for (int i = 0; i < ntotal; ++i) wr(out, a_in[i].data(), dim);
        for (int i = 0; i < ntotal; ++i) wr(out, Delta[i].Velocity, dim);
        for (int i = 0; i < ntotal; ++i) buf[i] = Delta[i].Density;
        wr(out, buf.data(), ntotal);
        for (int i = 0; i < ntotal; ++i) buf[i] = Delta[i].Energy;
        wr(out, buf.data(), ntotal);
        for (int i = 0; i < ntotal; ++i) wr(out, P[i].x, dim);
        for (int i = 0; i < ntotal; ++i) wr(out, P[i].v, dim);
        for (int i = 0; i < ntotal; ++i) buf[i] = P[i].Density;
        wr(out, buf.data(), ntotal);
        wr(out, &mx, 1);
        wr(out, &mean, 1);
        fclose(out);
    } catch (const mysph::Error& e) {
        std::cerr << e.what() << "\n";
        return 3;
    }
    return 0;
}
