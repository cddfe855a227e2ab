// mysph.hpp — a C++ host interface with the names, argument meaning and
// particle type of mySPH's module procedures, on top of the C ABI of
// libsphgpu (include/sph_gpu.h).
//
// The reference passes arrays of type(Particle) (src/Initialize/SPH.f90:6-25)
// to module procedures that mutate them: BGGS (asymmetricSearch.f90:160),
// con_density / sum_density (density.f90:10-107), divergence
// (divergence.f90:6), internal_force (internalForce.f90:10), external_force
// (externalForce.f90:7), arti_visc (artificialViscosity.f90:7),
// artificialStress (artificialTerm.f90:7), boundary (boundaryCondition.f90:15),
// courant_num (courantNumber.f90:7), single_step (singleStep.f90:1) and
// time_integration (timeIntegration.f90:22).  Here the particle system lives
// on the device inside a `Field`; each procedure runs there and writes its
// results back into the caller's Particle array as the reference would.
// Where the reference stops the program (`error stop`), these functions throw
// mysph::Error carrying the library status.
#pragma once

#include <array>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sph_gpu.h"

namespace mysph {

// type(Particle) of SPH.f90:6-25 (x, v, Displacement of Dim components;
// Stress column-major Dim x Dim; neighborList 1-based after BGGS).
struct Particle {
    int Type = 0, State = 0, Boundary = 0;
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, Displacement[3] = {0, 0, 0};
    double Mass = 0, Density = 0;
    double Pressure = 0, InternalEnergy = 0, SoundSpeed = 0, SmoothingLength = 0, Viscosity = 0;
    double divergencePosition = 0, divergenceVelocity = 0;
    double Stress[9] = {};
    int neighborNum = 0;
    std::vector<int> neighborList;
};

// type(Update) of SPH.f90:27-30.
struct Update {
    double Velocity[3] = {0, 0, 0};
    double Density = 0, Energy = 0;
};

using Vec = std::array<double, 3>;

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& where, const std::string& msg);
    int status;
};

// The device-resident particle system of P(1:ntotal+ndummy): real particles
// first, then the dummy (wall) particles, as in the reference.
class Field {
public:
    Field(const sph_params& prm, std::vector<Particle>& P, int ntotal, int ndummy,
          const std::vector<double>* shear = nullptr);
    ~Field();
    Field(const Field&) = delete;
    Field& operator=(const Field&) = delete;

    sph_ctx* ctx = nullptr;
    int Dim = 0, ntotal = 0, ndummy = 0;
    std::vector<Particle>& P;

    void check(int status, const char* where) const;
    void pull();                       // device state -> P (x, v, rho, p, e, c, Displacement, Stress, div)
    std::vector<double> field(int32_t id) const;
    double time() const;
    long long step() const;
};

void BGGS(Field& f);
void con_density(Field& f, int ntotal, std::vector<double>& drhodt);
void sum_density(Field& f, int ntotal);
void divergence(Field& f, int ntotal);
void internal_force(Field& f, int ntotal, std::vector<Vec>& dvdt, std::vector<double>& dedt);
void external_force(Field& f, int ntotal, std::vector<Vec>& dvdt);
void arti_visc(Field& f, int ntotal, std::vector<Vec>& dvdt, std::vector<double>& dedt);
void artificialStress(Field& f, int ntotal, std::vector<Vec>& dvdt);
// arti_heat (artificialHeat.f90:6-56): the artificial-heat energy rate
void arti_heat(Field& f, int ntotal, std::vector<double>& dedt);
void single_step(Field& f, int ntotal, std::vector<Update>& Delta);
// boundary (boundaryCondition.f90:15-45): fixedBoundary on Delta%Velocity
void boundary(Field& f, int ntotal, std::vector<Update>& Delta);
// courant_num (courantNumber.f90:7-31), elementwise over the three arrays
std::vector<double> courant_num(Field& f, const std::vector<double>& hsml, const std::vector<double>& div_v,
                                const std::vector<double>& c);
void time_integration(Field& f, long long nsteps, double& max_courant, double& aver_courant);
void print_statistics(Field& f, std::ostream& out);

}  // namespace mysph
