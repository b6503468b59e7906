// fields.h -- field and Poisson kernel launchers (host declarations).
#pragma once

#include <algorithm>

#include "circuit.hpp"
#include "common.cuh"

namespace pgd {

// Reduction layout shared by every deterministic sum: a block of 256 threads
// owns kChunk consecutive cells, thread t adds cells t, t+256, ... in order.
constexpr int kItems = 4;
constexpr int kChunk = 256 * kItems;

// Device-resident PCG scalars; every kernel of one solve reads and writes it.
// Chronopoulos-Gear form: rz = gamma = r.u, pq = delta = w.u.
struct PcgState {
    double rz, rr, bb, pq, beta, lim, mean, of_residual, alpha;
    int done, iters, converged, k;
    unsigned int ticket;
    unsigned int pad2[3];
};

// q * weight * 2^-kDepositBits per species (the FP32 form's fixed-point deposit).
struct SpeciesValues {
    int n;
    double v[PICGPU_MAX_SPECIES];
};

cudaError_t fields_set_patches(const PatchConst& p);
void launch_charge_update_mixed(const DMesh& m, int vw, const SpeciesValues& sv, const unsigned long long* acc9,
                                double* vtx, double space_charge, double* rho, cudaStream_t s);
void launch_corner_E(const DMesh& m, const double* E, const double* Ept, float4* Ec4, cudaStream_t s);
int pcg_blocks(int n);
void launch_charge_update(const DMesh& m, int vw, int fixed, double fix_scale, const double* ccd,
                          const double* vtxd, const long long* ccf, const long long* vtxf,
                          double space_charge, double* rho, cudaStream_t s);
void launch_floating_update(double* qconv, double* sigma, double* grad_bc, cudaStream_t s);

// Circuit model of a context (constant over a run).
struct CircuitParams {
    int model, anode, cathode, n_faces;
    const int* faces;     // the cathode's boundary faces, in face order
    double a[5];          // circuitRLC backward-difference coefficients
    double k;             // a0 * epsilon * cathode area
    double area;          // cathode area
    double I;             // IdealCurrentSource current
    double dt;
};
void launch_circuit_pre(const CircuitParams& P, double src, double* qconv, double* grad_bc, pg::CircuitState* S,
                        cudaStream_t s);
// Fowler-Nordheim current density summed over the given boundary faces -> *out.
void launch_fowler_nordheim(const DMesh& m, const double* Eb, const int* faces, int n, double W, double* out,
                            cudaStream_t s);
void launch_circuit_post(const CircuitParams& P, const DMesh& m, double src, double beta, const double* phi,
                         double* qconv, pg::CircuitState* S, cudaStream_t s);
void launch_rhs(const DMesh& m, const double* rho, const double* grad_bc, double* b, int singular,
                double* part, PcgState* st, cudaStream_t s);
// PCG (Chronopoulos-Gear form, Jacobi preconditioner).  part holds 4 x
// pcg_blocks(n) doubles; the state's ticket must be zero on entry.
void launch_pcg_init(const DMesh& m, const double* b, const double* x, double* r, double* u, double* w,
                     double* part, PcgState* st, double tol, cudaStream_t s);
void launch_pcg_iteration(const DMesh& m, double* x, double* r, double* u, double* w, double* p, double* sv,
                          double* part, PcgState* st, int maxit, cudaStream_t s);
void launch_of_residual(const DMesh& m, const double* b, const double* x, double* part, PcgState* st,
                        cudaStream_t s);
void launch_efield(const DMesh& m, const double* phi, const double* grad_bc, double* E, double* Eb,
                   double* Ept, float* E32, float* Ept32, cudaStream_t s);
void launch_to_float(const double* a, float* b, long n, cudaStream_t s);
void launch_fill(double* a, long n, double v, cudaStream_t s);
void launch_diagnostics(const int32_t* tet, const double* u0, const double* u1, const double* u2,
                        const float* f0, const float* f1, const float* f2, int n, double mass,
                        double weight, const double* nw, double* out, cudaStream_t s);
void launch_field_energy(const double* E, const double* vol, int n, double* out, cudaStream_t s);

}  // namespace pgd
