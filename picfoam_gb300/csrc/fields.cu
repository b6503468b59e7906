// fields.cu -- charge density, electrostatic Poisson PCG and the E field.
//
// Built with --fmad=false: each kernel evaluates in the order of the CPU
// oracle, and every reduction runs in one fixed tree order (256 threads,
// kItems strided items per thread; lane l of warp 0 adds threads l, l+32, ...,
// l+224, then a warp xor-tree; the last block of a launch combines the block
// partials in the same order), so the FP64 Poisson solve is bit-reproducible
// and matches the oracle bit for bit.
//
//   charge_update   ChargeDistribution::update (VolumeWeighting.C:138-164,
//                   CellAverage.C:63-68) + spaceCharge (PICCloud.C:687-690)
//   rhs + pcg_*     solve(fvm::laplacian(phiE) + rhoCharge/epsilon0)
//                   (ElectroStaticSolver.C:61-64), PCG with a Jacobi
//                   preconditioner on the SPD operator -laplacian
//   grad_E          E = -fvc::grad(phiE), Gauss linear (ElectroStaticSolver.C:68)
//   boundary_E      corrected boundary values of E
//   point_E         cell -> point interpolation (VolumeWeightingFW.C:70-75)
#include "circuit.hpp"
#include "emission.hpp"
#include "fields.h"
#include "reduce.cuh"

#include <algorithm>

namespace pgd {

__constant__ PatchConst c_patchF;

constexpr double kMu0 = 4.0 * kPi * 1e-7;
__device__ __forceinline__ double eps0() { return 1.0 / (kMu0 * kC * kC); }

// ------------------------------------------------------------ charge -----
__global__ void charge_update_kernel(DMesh m, int volume_weighting, int fixed, double fix_scale,
                                     const double* __restrict__ ccd, const double* __restrict__ vtxd,
                                     const long long* __restrict__ ccf,
                                     const long long* __restrict__ vtxf, double space_charge,
                                     double* __restrict__ rho) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const double V = m.vol[c];
    const double ccv = fixed ? double(ccf[c]) / fix_scale : ccd[c];
    double r = 0.0;
    if (!volume_weighting) {
        r = ccv / V;
    } else {
        r = r + ccv / V;
        for (int q = 0; q < 8; ++q) {
            const int pt = m.cell_pt[8 * size_t(c) + q];
            const double vv = fixed ? double(vtxf[pt]) / fix_scale : vtxd[pt];
            r = r + (m.vw_weight[8 * size_t(c) + q] * vv) / V;
        }
    }
    rho[c] = r + space_charge;
}

// Charge update of the FP32 form.  The move kernel leaves per species and
// cell 9 fixed-point slots (centre + 8 corners); a point's charge is the
// integer sum of the corner slots of every cell around it (syncPointData of
// VolumeWeighting.C:141-146, cyclic images included), times q w 2^-kDepositBits.
__global__ void point_charge_kernel(DMesh m, SpeciesValues sv, const unsigned long long* __restrict__ acc9,
                                    double* __restrict__ vtx) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.n_points) return;
    const size_t stride = 9 * size_t(m.n_cells);
    double v = 0.0;
    for (int s = 0; s < sv.n; ++s) {
        unsigned long long sum = 0;
        for (int k = m.pc_start[p]; k < m.pc_start[p + 1]; ++k) sum += acc9[s * stride + m.pc_slot[k]];
        v += sv.v[s] * double(sum);
    }
    vtx[p] = v;
}

__global__ void charge_update_mixed_kernel(DMesh m, int volume_weighting, SpeciesValues sv,
                                           const unsigned long long* __restrict__ acc9,
                                           const double* __restrict__ vtx, double space_charge,
                                           double* __restrict__ rho) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const size_t stride = 9 * size_t(m.n_cells);
    const double V = m.vol[c];
    double ccv = 0.0;
    for (int s = 0; s < sv.n; ++s) ccv += sv.v[s] * double(acc9[s * stride + 9 * size_t(c)]);
    // one division per cell: the FP32 form's density is compared with the
    // oracle within its tolerance, and FP64 divisions are the cost here
    if (volume_weighting)
        for (int q = 0; q < 8; ++q) ccv += m.vw_weight[8 * size_t(c) + q] * vtx[m.cell_pt[8 * size_t(c) + q]];
    rho[c] = ccv / V + space_charge;
}

void launch_charge_update_mixed(const DMesh& m, int vw, const SpeciesValues& sv, const unsigned long long* acc9,
                                double* vtx, double space_charge, double* rho, cudaStream_t s) {
    if (vw) point_charge_kernel<<<(m.n_points + 255) / 256, 256, 0, s>>>(m, sv, acc9, vtx);
    charge_update_mixed_kernel<<<(m.n_cells + 255) / 256, 256, 0, s>>>(m, vw, sv, acc9, vtx, space_charge, rho);
}

// E per cell for the FP32 move kernel: centre value + the 8 corner (point)
// values as float4, so a particle's field gather reads one cell block.
__global__ void corner_E_kernel(DMesh m, const double* __restrict__ E, const double* __restrict__ Ept,
                                float4* __restrict__ Ec4) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const double* e = E + 3 * size_t(c);
    Ec4[9 * size_t(c)] = make_float4(float(e[0]), float(e[1]), float(e[2]), 0.f);
    for (int q = 0; q < 8; ++q) {
        const double* p = Ept + 3 * size_t(m.cell_pt[8 * size_t(c) + q]);
        Ec4[9 * size_t(c) + 1 + q] = make_float4(float(p[0]), float(p[1]), float(p[2]), 0.f);
    }
}

void launch_corner_E(const DMesh& m, const double* E, const double* Ept, float4* Ec4, cudaStream_t s) {
    corner_E_kernel<<<(m.n_cells + 255) / 256, 256, 0, s>>>(m, E, Ept, Ec4);
}

// FloatingPotential::preUpdate_Boundary (FloatingPotential.C:89-100)
__global__ void floating_update_kernel(double* qconv, double* sigma, double* grad_bc) {
    const int p = threadIdx.x;
    if (p >= c_patchF.n || c_patchF.kind[p] != PICGPU_PATCH_FLOATING) return;
    sigma[p] += qconv[p] / c_patchF.area[p];
    grad_bc[p] = sigma[p] / eps0();
    qconv[p] = 0.0;
}

// Circuit models: preUpdate_Boundary before the solve, postUpdate_Boundary
// after it (PICCloud.C:1457-1464).  One thread / one block of
// pg::kCircuitLanes lanes; the lane order of the cathode-face sum is the one
// pg::circuit_face_sum restates.
__global__ void circuit_pre_kernel(CircuitParams P, double src, double* qconv, double* grad_bc,
                                   pg::CircuitState* S) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    pg::CircuitState st = *S;
    pg::circuit_pre_update(P.model, P.cathode, P.a, P.area, P.I, P.dt, eps0(), src, qconv, grad_bc, st);
    *S = st;
}

__global__ void __launch_bounds__(pg::kCircuitLanes)
circuit_post_kernel(CircuitParams P, DMesh m, double src, double beta, const double* __restrict__ phi,
                    double* qconv, pg::CircuitState* S) {
    __shared__ double lane[pg::kCircuitLanes];
    const int t = threadIdx.x;
    double a = 0.0;
    if (P.model == PICGPU_CIRCUIT_RLC) {
        for (int i = t; i < P.n_faces; i += pg::kCircuitLanes) {
            const int b = P.faces[i];
            a = a + pg::face_value(pg::kRuleRlc, 0.0, 0.0, P.k, m.bf_delta[b], phi[m.bf_cell[b]]);
        }
    } else if (P.model == PICGPU_CIRCUIT_IDEAL_CURRENT) {
        for (int i = t; i < P.n_faces; i += pg::kCircuitLanes) {
            const int b = P.faces[i];
            a = a + m.bf_area[b] * phi[m.bf_cell[b]];
        }
    }
    lane[t] = a;
    __syncthreads();
    for (int s = pg::kCircuitLanes / 2; s > 0; s >>= 1) {
        if (t < s) lane[t] = lane[t] + lane[t + s];
        __syncthreads();
    }
    if (t != 0) return;
    pg::CircuitState st = *S;
    pg::circuit_post_update(P.model, P.anode, P.cathode, P.n_faces, P.a, P.area, P.dt, src, beta, lane[0], qconv,
                            st);
    *S = st;
}

// FowlerNordheim::emission (FowlerNordheim.C:64-86): the current density
// summed over the patch faces, in the lane order pg::emission_face_sum
// restates.
__global__ void __launch_bounds__(pg::kEmissionLanes)
fowler_nordheim_kernel(DMesh m, const double* __restrict__ Eb, const int* __restrict__ faces, int n, double W,
                       double* out) {
    __shared__ double lane[pg::kEmissionLanes];
    const int t = threadIdx.x;
    double a = 0.0;
    for (int i = t; i < n; i += pg::kEmissionLanes) {
        const int b = faces[i];
        a = a + pg::fowler_nordheim_face(Eb + 3 * size_t(b), m.bf_normal + 3 * size_t(b), W);
    }
    lane[t] = a;
    __syncthreads();
    for (int s = pg::kEmissionLanes / 2; s > 0; s >>= 1) {
        if (t < s) lane[t] = lane[t] + lane[t + s];
        __syncthreads();
    }
    if (t == 0) *out = lane[0];
}

// ----------------------------------------------------------- Poisson -----
__global__ void rhs_kernel(DMesh m, const double* __restrict__ rho, const double* __restrict__ grad_bc,
                           double* __restrict__ b) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    double t = (rho[c] / eps0()) * m.vol[c];
    for (int f = 0; f < 6; ++f) {
        const int bf = m.cell_bface[6 * size_t(c) + f];
        if (bf < 0) continue;
        const int pa = m.bf_patch[bf];
        const int rule = pg::face_rule(c_patchF.kind[pa], c_patchF.phi_bc[pa]);
        if (rule != pg::kRuleNone)
            t = t + pg::face_rhs(rule, c_patchF.phi[pa], grad_bc[pa], c_patchF.rlc_k[pa], m.bf_area[bf],
                                 m.bf_delta[bf]);
    }
    b[c] = t;
}

__global__ void __launch_bounds__(256) sum_kernel(const double* __restrict__ v, int n,
                                                  double* part, PcgState* st) {
    __shared__ double ws[256];
    double s = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) s = s + v[i];
    }
    const double bs = block_tree(s, ws);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (arrive_last(&st->ticket)) {
        const double tot = final_sum(part, gridDim.x, ws);
        if (threadIdx.x == 0) st->mean = tot / double(n);
    }
}

__global__ void sub_mean_kernel(double* b, int n, const PcgState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = b[i] - st->mean;
}

// y = M x in the row of cell c.  On a uniform block mesh every coupled face
// in direction f carries the same coefficient (the mesh builder computes it
// from the one geometry class; the host checks every face), so the per-face
// array is not read.
template <bool Uniform>
__device__ __forceinline__ double apply_M(const DMesh& m, const double* __restrict__ x, int c) {
    double s = m.Mdiag[c] * x[c];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const int nb = m.nbr[6 * size_t(c) + f];
        if (nb >= 0) s = fma(Uniform ? m.lap_coef[f] : m.Moff[6 * size_t(c) + f], x[nb], s);
    }
    return s;
}

// The PCG runs in the Chronopoulos-Gear form (one reduction point per
// iteration): with u = D^-1 r, w = M u, s = M p,
//   p = u + beta p,  s = w + beta s,  x += alpha p,  r -= alpha s,  u = D^-1 r
//   w = M u,  gamma = r.u,  delta = w.u,  beta = gamma / gamma_old,
//   alpha = gamma / (delta - beta gamma / alpha_old).
// It is the same Krylov iteration as the textbook PCG of lduMatrix (the
// iterates agree in exact arithmetic) with one global synchronisation per
// iteration instead of two and no per-thread division.  The vector updates,
// the SpMV and the dot products use explicit fused multiply-adds (the oracle
// calls std::fma at the same places): FP64 issue is the bound of both kernels
// on this part, and a fused a*b + c is one FP64 instruction instead of two.

// r = b - M x, u = D^-1 r; partials of gamma = r.u, r.r and b.b.
template <bool Uniform>
__global__ void __launch_bounds__(256) pcg_init_kernel(DMesh m, const double* __restrict__ b,
                                                       const double* __restrict__ x, double* __restrict__ r,
                                                       double* __restrict__ u, double* part) {
    __shared__ double ws[256];
    const int n = m.n_cells;
    const int nb = gridDim.x;
    double sg = 0.0, srr = 0.0, sbb = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const double mx = apply_M<Uniform>(m, x, int(i));
            const double ri = b[i] - mx;
            const double ui = m.dinv[i] * ri;
            r[i] = ri;
            u[i] = ui;
            sg = fma(ri, ui, sg);
            srr = fma(ri, ri, srr);
            sbb = fma(b[i], b[i], sbb);
        }
    }
    const double b0 = block_tree(sg, ws);
    const double b1 = block_tree(srr, ws);
    const double b2 = block_tree(sbb, ws);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b0;
        part[nb + blockIdx.x] = b1;
        part[3 * nb + blockIdx.x] = b2;
    }
}

// w = M u; partial delta = w.u.  The last block finalises: after the
// initialisation (init = 1) it sets alpha_0, otherwise it closes iteration
// k + 1 (convergence test on r.r, then beta and alpha).
template <bool Uniform>
__global__ void __launch_bounds__(256) pcg_spmv_kernel(DMesh m, const double* __restrict__ u,
                                                       double* __restrict__ w, double* part, PcgState* st,
                                                       int init, double tol, int maxit) {
    if (!init && st->done) return;
    __shared__ double ws[256];
    const int n = m.n_cells;
    const int nb = gridDim.x;
    double sd = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const double wi = apply_M<Uniform>(m, u, int(i));
            w[i] = wi;
            sd = fma(wi, u[i], sd);
        }
    }
    const double b2 = block_tree(sd, ws);
    if (threadIdx.x == 0) part[2 * nb + blockIdx.x] = b2;
    if (arrive_last(&st->ticket)) {
        const double g = final_sum(part, nb, ws);
        const double rr = final_sum(part + nb, nb, ws);
        const double d = final_sum(part + 2 * nb, nb, ws);
        const double bb = init ? final_sum(part + 3 * nb, nb, ws) : 0.0;
        if (threadIdx.x == 0) {
            if (init) {
                st->rz = g;
                st->rr = rr;
                st->bb = bb;
                st->pq = d;
                st->lim = (tol * tol) * bb;
                st->alpha = g / d;
                st->beta = 0.0;
                st->iters = 0;
                st->k = 0;
                st->done = rr <= st->lim ? 1 : 0;
                st->converged = st->done;
            } else {
                const int k = st->k + 1;
                st->rr = rr;
                st->pq = d;
                st->k = k;
                st->iters = k;
                if (rr <= st->lim) {
                    st->done = 1;
                    st->converged = 1;
                } else if (k >= maxit) {
                    st->done = 1;
                    st->converged = 0;
                } else {
                    const double beta = g / st->rz;
                    st->alpha = g / (d - beta * g / st->alpha);
                    st->beta = beta;
                    st->rz = g;
                }
            }
        }
    }
}

// p = u + beta p, s = w + beta s (p = u, s = w on the first iteration),
// x += alpha p, r -= alpha s, u = D^-1 r; partials of gamma = r.u and r.r.
__global__ void __launch_bounds__(256) pcg_update_kernel(DMesh m, double* __restrict__ x, double* __restrict__ r,
                                                         double* __restrict__ u, const double* __restrict__ w,
                                                         double* __restrict__ p, double* __restrict__ sv,
                                                         double* part, PcgState* st) {
    if (st->done) return;
    __shared__ double ws[256];
    const int n = m.n_cells;
    const int nb = gridDim.x;
    const int first = st->k == 0;
    const double alpha = st->alpha, beta = st->beta;
    double sg = 0.0, srr = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            double pi, si;
            if (first) {
                pi = u[i];
                si = w[i];
            } else {
                pi = fma(beta, p[i], u[i]);
                si = fma(beta, sv[i], w[i]);
            }
            p[i] = pi;
            sv[i] = si;
            x[i] = fma(alpha, pi, x[i]);
            const double ri = fma(-alpha, si, r[i]);
            const double ui = m.dinv[i] * ri;
            r[i] = ri;
            u[i] = ui;
            sg = fma(ri, ui, sg);
            srr = fma(ri, ri, srr);
        }
    }
    const double b0 = block_tree(sg, ws);
    const double b1 = block_tree(srr, ws);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b0;
        part[nb + blockIdx.x] = b1;
    }
}

// OpenFOAM-normalised residual terms (reported, not used for convergence).
__global__ void __launch_bounds__(256) of_residual_kernel(DMesh m, const double* __restrict__ b,
                                                          const double* __restrict__ x, double* part,
                                                          PcgState* st) {
    __shared__ double ws[256];
    const double mean = st->mean;
    const int n = m.n_cells;
    const int nb = gridDim.x;
    double sn = 0.0, sd = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const double ax = apply_M<false>(m, x, int(i));
            double rowsum = m.Mdiag[i];
            for (int f = 0; f < 6; ++f)
                if (m.nbr[6 * size_t(i) + f] >= 0) rowsum += m.Moff[6 * size_t(i) + f];
            const double axr = rowsum * mean;
            sn += fabs(b[i] - ax);
            sd += fabs(ax - axr) + fabs(b[i] - axr);
        }
    }
    const double b0 = block_tree(sn, ws);
    const double b1 = block_tree(sd, ws);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b0;
        part[nb + blockIdx.x] = b1;
    }
    if (arrive_last(&st->ticket)) {
        const double num = final_sum(part, nb, ws);
        const double den = final_sum(part + nb, nb, ws);
        if (threadIdx.x == 0) st->of_residual = num / (den + 1e-20);
    }
}

// ------------------------------------------------------------ E field ----
__global__ void grad_E_kernel(DMesh m, const double* __restrict__ phi,
                              const double* __restrict__ grad_bc, double* __restrict__ E) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const int cl = m.cell_class[c];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int f = 0; f < 6; ++f) {
        const int nb = m.nbr[6 * size_t(c) + f];
        double pf;
        if (nb >= 0) {
            const double w = m.ip_weight[6 * size_t(c) + f];
            pf = w * phi[c] + (1.0 - w) * phi[nb];
        } else {
            const int bf = m.cell_bface[6 * size_t(c) + f];
            if (bf < 0) continue;
            const int pa = m.bf_patch[bf];
            pf = pg::face_value(pg::face_rule(c_patchF.kind[pa], c_patchF.phi_bc[pa]), c_patchF.phi[pa],
                                grad_bc[pa], c_patchF.rlc_k[pa], m.bf_delta[bf], phi[c]);
        }
        const double area = m.farea[size_t(cl) * 6 + f];
        const double* n = m.fnormal + size_t(cl) * 18 + 3 * f;
        g0 = g0 + pf * (n[0] * area);
        g1 = g1 + pf * (n[1] * area);
        g2 = g2 + pf * (n[2] * area);
    }
    const double V = m.vol[c];
    E[3 * size_t(c)] = -(g0 / V);
    E[3 * size_t(c) + 1] = -(g1 / V);
    E[3 * size_t(c) + 2] = -(g2 / V);
}

__global__ void boundary_E_kernel(DMesh m, const double* __restrict__ phi,
                                  const double* __restrict__ grad_bc, const double* __restrict__ E,
                                  double* __restrict__ Eb) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m.n_bfaces) return;
    const int c = m.bf_cell[b];
    const int pa = m.bf_patch[b];
    const double* Ec = E + 3 * size_t(c);
    const double* n = m.bf_normal + 3 * size_t(b);
    const double sn = pg::face_sn_grad(pg::face_rule(c_patchF.kind[pa], c_patchF.phi_bc[pa]), c_patchF.phi[pa],
                                       grad_bc[pa], c_patchF.rlc_k[pa], m.bf_delta[b], phi[c]);
    const double En = Ec[0] * n[0] + Ec[1] * n[1] + Ec[2] * n[2];
    for (int a = 0; a < 3; ++a) Eb[3 * size_t(b) + a] = (Ec[a] - En * n[a]) - sn * n[a];
}

__global__ void point_E_kernel(DMesh m, const double* __restrict__ E, const double* __restrict__ Eb,
                               double* __restrict__ Ept, float* __restrict__ Ept32) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.n_points) return;
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    for (int k = m.pi_start[p]; k < m.pi_start[p + 1]; ++k) {
        const int s = m.pi_src[k];
        const double* src = s >= 0 ? E + 3 * size_t(s) : Eb + 3 * size_t(-s - 1);
        const double w = m.pi_w[k];
        e0 = e0 + w * src[0];
        e1 = e1 + w * src[1];
        e2 = e2 + w * src[2];
    }
    Ept[3 * size_t(p)] = e0;
    Ept[3 * size_t(p) + 1] = e1;
    Ept[3 * size_t(p) + 2] = e2;
    Ept32[3 * size_t(p)] = float(e0);
    Ept32[3 * size_t(p) + 1] = float(e1);
    Ept32[3 * size_t(p) + 2] = float(e2);
}

__global__ void to_float_kernel(const double* __restrict__ a, float* __restrict__ b, long n) {
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) b[i] = float(a[i]);
}

__global__ void fill_kernel(double* a, long n, double v) {
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// ------------------------------------------------------- diagnostics -----
__global__ void diagnostics_kernel(const int32_t* __restrict__ tet, const double* __restrict__ u0,
                                   const double* __restrict__ u1, const double* __restrict__ u2,
                                   const float* __restrict__ f0, const float* __restrict__ f1,
                                   const float* __restrict__ f2, int n, double mass, double species_weight,
                                   const double* __restrict__ nw, double* out /* 10 */) {
    double ke = 0, ker = 0, mx = 0, my = 0, mz = 0, vx = 0, vy = 0, vz = 0, w = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (tet[i] < 0) continue;
        const double weight = nw ? nw[i] : species_weight;   // the parcel's nParticle
        const double a = u0 ? u0[i] : double(f0[i]);
        const double b = u0 ? u1[i] : double(f1[i]);
        const double c = u0 ? u2[i] : double(f2[i]);
        const double uu = a * a + b * b + c * c;
        ke += 0.5 * mass * uu * weight;
        const double be = sqrt(uu) / kC;
        ker += (1.0 / sqrt(1.0 - be * be) - 1.0) * mass * kC * kC;
        mx += weight * mass * a;
        my += weight * mass * b;
        mz += weight * mass * c;
        vx += weight * a * a;
        vy += weight * b * b;
        vz += weight * c * c;
        w += weight;
    }
    double vals[9] = {ke, ker, mx, my, mz, vx, vy, vz, w};
    for (int k = 0; k < 9; ++k) {
        double v = vals[k];
        for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(out + k, v);
    }
}

__global__ void field_energy_kernel(const double* __restrict__ E, const double* __restrict__ vol, int n,
                                    double* out) {
    double s = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const double* e = E + 3 * size_t(c);
        s += (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * vol[c];
    }
    for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(out, s);
}

// ------------------------------------------------------------ launchers --
static inline int blocks(long n, int bs) { return int((n + bs - 1) / bs); }

cudaError_t fields_set_patches(const PatchConst& p) {
    return cudaMemcpyToSymbol(c_patchF, &p, sizeof p);
}

void launch_charge_update(const DMesh& m, int vw, int fixed, double fix_scale, const double* ccd,
                          const double* vtxd, const long long* ccf, const long long* vtxf,
                          double space_charge, double* rho, cudaStream_t s) {
    charge_update_kernel<<<blocks(m.n_cells, 256), 256, 0, s>>>(m, vw, fixed, fix_scale, ccd, vtxd, ccf,
                                                                vtxf, space_charge, rho);
}

void launch_floating_update(double* qconv, double* sigma, double* grad_bc, cudaStream_t s) {
    floating_update_kernel<<<1, 32, 0, s>>>(qconv, sigma, grad_bc);
}

void launch_circuit_pre(const CircuitParams& P, double src, double* qconv, double* grad_bc, pg::CircuitState* S,
                        cudaStream_t s) {
    circuit_pre_kernel<<<1, 32, 0, s>>>(P, src, qconv, grad_bc, S);
}

void launch_circuit_post(const CircuitParams& P, const DMesh& m, double src, double beta, const double* phi,
                         double* qconv, pg::CircuitState* S, cudaStream_t s) {
    circuit_post_kernel<<<1, pg::kCircuitLanes, 0, s>>>(P, m, src, beta, phi, qconv, S);
}

void launch_fowler_nordheim(const DMesh& m, const double* Eb, const int* faces, int n, double W, double* out,
                            cudaStream_t s) {
    fowler_nordheim_kernel<<<1, pg::kEmissionLanes, 0, s>>>(m, Eb, faces, n, W, out);
}

int pcg_blocks(int n) { return (n + kChunk - 1) / kChunk; }

void launch_rhs(const DMesh& m, const double* rho, const double* grad_bc, double* b, int singular,
                double* part, PcgState* st, cudaStream_t s) {
    rhs_kernel<<<blocks(m.n_cells, 256), 256, 0, s>>>(m, rho, grad_bc, b);
    if (singular) {
        sum_kernel<<<pcg_blocks(m.n_cells), 256, 0, s>>>(b, m.n_cells, part, st);
        sub_mean_kernel<<<blocks(m.n_cells, 256), 256, 0, s>>>(b, m.n_cells, st);
    }
}

void launch_pcg_init(const DMesh& m, const double* b, const double* x, double* r, double* u, double* w,
                     double* part, PcgState* st, double tol, cudaStream_t s) {
    const int nb = pcg_blocks(m.n_cells);
    if (m.lap_uniform) {
        pcg_init_kernel<true><<<nb, 256, 0, s>>>(m, b, x, r, u, part);
        pcg_spmv_kernel<true><<<nb, 256, 0, s>>>(m, u, w, part, st, 1, tol, 0);
    } else {
        pcg_init_kernel<false><<<nb, 256, 0, s>>>(m, b, x, r, u, part);
        pcg_spmv_kernel<false><<<nb, 256, 0, s>>>(m, u, w, part, st, 1, tol, 0);
    }
}

void launch_pcg_iteration(const DMesh& m, double* x, double* r, double* u, double* w, double* p, double* sv,
                          double* part, PcgState* st, int maxit, cudaStream_t s) {
    const int nb = pcg_blocks(m.n_cells);
    pcg_update_kernel<<<nb, 256, 0, s>>>(m, x, r, u, w, p, sv, part, st);
    if (m.lap_uniform) pcg_spmv_kernel<true><<<nb, 256, 0, s>>>(m, u, w, part, st, 0, 0.0, maxit);
    else pcg_spmv_kernel<false><<<nb, 256, 0, s>>>(m, u, w, part, st, 0, 0.0, maxit);
}

void launch_of_residual(const DMesh& m, const double* b, const double* x, double* part, PcgState* st,
                        cudaStream_t s) {
    sum_kernel<<<pcg_blocks(m.n_cells), 256, 0, s>>>(x, m.n_cells, part, st);
    of_residual_kernel<<<pcg_blocks(m.n_cells), 256, 0, s>>>(m, b, x, part, st);
}

void launch_efield(const DMesh& m, const double* phi, const double* grad_bc, double* E, double* Eb,
                   double* Ept, float* E32, float* Ept32, cudaStream_t s) {
    grad_E_kernel<<<blocks(m.n_cells, 256), 256, 0, s>>>(m, phi, grad_bc, E);
    if (m.n_bfaces > 0) boundary_E_kernel<<<blocks(m.n_bfaces, 256), 256, 0, s>>>(m, phi, grad_bc, E, Eb);
    point_E_kernel<<<blocks(m.n_points, 256), 256, 0, s>>>(m, E, Eb, Ept, Ept32);
    to_float_kernel<<<blocks(3L * m.n_cells, 256), 256, 0, s>>>(E, E32, 3L * m.n_cells);
}

void launch_to_float(const double* a, float* b, long n, cudaStream_t s) {
    to_float_kernel<<<blocks(n, 256), 256, 0, s>>>(a, b, n);
}

void launch_fill(double* a, long n, double v, cudaStream_t s) {
    if (n > 0) fill_kernel<<<blocks(n, 256), 256, 0, s>>>(a, n, v);
}

void launch_diagnostics(const int32_t* tet, const double* u0, const double* u1, const double* u2,
                        const float* f0, const float* f1, const float* f2, int n, double mass,
                        double weight, const double* nw, double* out, cudaStream_t s) {
    if (n <= 0) return;
    diagnostics_kernel<<<std::min(blocks(n, 256), 1216), 256, 0, s>>>(tet, u0, u1, u2, f0, f1, f2, n, mass,
                                                                       weight, nw, out);
}

void launch_field_energy(const double* E, const double* vol, int n, double* out, cudaStream_t s) {
    field_energy_kernel<<<std::min(blocks(n, 256), 1216), 256, 0, s>>>(E, vol, n, out);
}

}  // namespace pgd
