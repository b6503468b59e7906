// mg.cu -- flexible FP64 PCG with an FP32 aggregation-multigrid V-cycle as
// preconditioner (the role of OpenFOAM's GAMG preconditioner inside PCG; the
// solver call it replaces is ElectroStaticSolver.C:61-64).
//
// Kernels, all deterministic (no atomics in any sum):
//   mg_init      r = b - M x, r.r and b.b; r as FP32 into the level-0 voxels
//   V-cycle      per level: Jacobi sweeps, residual + restriction to the
//                aggregates, (coarse level), prolongation, Jacobi sweeps;
//                dense inverse times vector on the coarsest level
//   mg_gather    z = V-cycle result, r.z and r.z_old -> beta
//   mg_direction p = z + beta p
//   mg_spmv      q = M p, p.q -> alpha
//   mg_axpy      x += alpha p, r -= alpha q, r.r -> convergence; r into level 0
// Every kernel after the initialisation returns at once when the solve is
// done, so a CUDA graph of a fixed number of iterations stops exactly at
// convergence.
#include "mg.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>

#include "fields.h"
#include "reduce.cuh"

namespace pgd {

namespace {

constexpr int kGraphIters = 8;

// Level description passed by value to the FP32 kernels.
struct Lv {
    int X, Y, Z, cx, cy, cz;
    long V;
    int uniform;
    float coef[6];
    const float* __restrict__ diag;
    const float* __restrict__ inv;
    const float* __restrict__ off;
};

Lv view(const MgLevel& L) {
    Lv v{};
    v.X = L.n[0];
    v.Y = L.n[1];
    v.Z = L.n[2];
    v.cx = L.cyc[0];
    v.cy = L.cyc[1];
    v.cz = L.cyc[2];
    v.V = L.V;
    v.uniform = L.uniform;
    for (int f = 0; f < 6; ++f) v.coef[f] = L.coef[f];
    v.diag = L.diag;
    v.inv = L.inv;
    v.off = L.off;
    return v;
}

// (A x)_v on one level.  A neighbour across a non-periodic edge has no
// coupling (its coefficient is zero, the index falls back to v itself); a
// hole neighbour holds zero, so the uniform form may use coef[f] there.
template <bool Uniform>
__device__ __forceinline__ float apply_A(const Lv& L, const float* __restrict__ x, long v, int i, int j, int k) {
    const long X = L.X, XY = long(L.X) * L.Y;
    long nb[6];
    bool ok[6];
    ok[0] = i > 0 || L.cx;
    nb[0] = i > 0 ? v - 1 : (L.cx ? v + X - 1 : v);
    ok[1] = i < L.X - 1 || L.cx;
    nb[1] = i < L.X - 1 ? v + 1 : (L.cx ? v - (X - 1) : v);
    ok[2] = j > 0 || L.cy;
    nb[2] = j > 0 ? v - X : (L.cy ? v + XY - X : v);
    ok[3] = j < L.Y - 1 || L.cy;
    nb[3] = j < L.Y - 1 ? v + X : (L.cy ? v - (XY - X) : v);
    ok[4] = k > 0 || L.cz;
    nb[4] = k > 0 ? v - XY : (L.cz ? v + L.V - XY : v);
    ok[5] = k < L.Z - 1 || L.cz;
    nb[5] = k < L.Z - 1 ? v + XY : (L.cz ? v - (L.V - XY) : v);
    float s = L.diag[v] * x[v];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const float a = Uniform ? (ok[f] ? L.coef[f] : 0.f) : L.off[f * L.V + v];
        s = fmaf(a, x[nb[f]], s);
    }
    return s;
}

__device__ __forceinline__ void decode(const Lv& L, long v, int& i, int& j, int& k) {
    i = int(v % L.X);
    const long r = v / L.X;
    j = int(r % L.Y);
    k = int(r / L.Y);
}

// First sweep from a zero guess: y = omega D^-1 b.
__global__ void __launch_bounds__(256) mg_smooth0_kernel(Lv L, const float* __restrict__ b, float* __restrict__ y,
                                                         float omega, const MgScalars* sc) {
    if (sc->done) return;
    const long v = long(blockIdx.x) * 256 + threadIdx.x;
    if (v >= L.V) return;
    y[v] = (omega * L.inv[v]) * b[v];
}

// One weighted-Jacobi sweep: y = x + omega D^-1 (b - A x).
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_smooth_kernel(Lv L, const float* __restrict__ b,
                                                        const float* __restrict__ x, float* __restrict__ y,
                                                        float omega, const MgScalars* sc) {
    if (sc->done) return;
    const long v = long(blockIdx.x) * 256 + threadIdx.x;
    if (v >= L.V) return;
    int i, j, k;
    decode(L, v, i, j, k);
    const float ax = apply_A<Uniform>(L, x, v, i, j, k);
    y[v] = fmaf(omega * L.inv[v], b[v] - ax, x[v]);
}

// Coarse right-hand side: bc[I] = sum over the active children of I of
// (b - A x), children in x-fastest order.
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_restrict_kernel(Lv F, Lv Cl, int fx, int fy, int fz,
                                                          const float* __restrict__ b, const float* __restrict__ x,
                                                          float* __restrict__ bc, const MgScalars* sc) {
    if (sc->done) return;
    const long I = long(blockIdx.x) * 256 + threadIdx.x;
    if (I >= Cl.V) return;
    int ci, cj, ck;
    decode(Cl, I, ci, cj, ck);
    float s = 0.f;
    for (int dz = 0; dz < fz; ++dz) {
        const int k = fz * ck + dz;
        if (k >= F.Z) break;
        for (int dy = 0; dy < fy; ++dy) {
            const int j = fy * cj + dy;
            if (j >= F.Y) break;
            for (int dx = 0; dx < fx; ++dx) {
                const int i = fx * ci + dx;
                if (i >= F.X) break;
                const long v = i + long(F.X) * (j + long(F.Y) * k);
                if (F.inv[v] != 0.f) s += b[v] - apply_A<Uniform>(F, x, v, i, j, k);
            }
        }
    }
    bc[I] = s;
}

// x += scale * xc[parent] on the active voxels.
__global__ void __launch_bounds__(256) mg_prolong_kernel(Lv F, int CX, int CY, int fx, int fy, int fz,
                                                         const float* __restrict__ xc, float* __restrict__ x,
                                                         float scale, const MgScalars* sc) {
    if (sc->done) return;
    const long v = long(blockIdx.x) * 256 + threadIdx.x;
    if (v >= F.V) return;
    if (F.inv[v] == 0.f) return;
    int i, j, k;
    decode(F, v, i, j, k);
    const long I = i / fx + long(CX) * (j / fy + long(CY) * (k / fz));
    x[v] = fmaf(scale, xc[I], x[v]);
}

// Coarsest level: x[idx[r]] = sum_k inv[r][k] b[idx[k]], one warp per row,
// lane l adds k = l, l + 32, ... then an xor-tree.
__global__ void __launch_bounds__(256) mg_coarse_kernel(const float* __restrict__ inv, const int* __restrict__ idx,
                                                        int nc, const float* __restrict__ b, float* __restrict__ x,
                                                        const MgScalars* sc) {
    if (sc->done) return;
    const int row = int((long(blockIdx.x) * 256 + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= nc) return;
    const float* a = inv + long(row) * nc;
    float s = 0.f;
    for (int k = lane; k < nc; k += 32) s = fmaf(a[k], b[idx[k]], s);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[idx[row]] = s;
}

// ---------------------------------------------------------- FP64 PCG -----
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

template <bool Uniform>
__global__ void __launch_bounds__(256) mg_init_kernel(DMesh m, const double* __restrict__ b,
                                                      const double* __restrict__ x, double* __restrict__ r,
                                                      const int* __restrict__ vox, float* __restrict__ b0,
                                                      double* part, MgScalars* sc, double tol, int maxit) {
    __shared__ double ws[256];
    const int n = m.n_cells;
    const int nb = gridDim.x;
    double srr = 0.0, sbb = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const double ri = b[i] - apply_M<Uniform>(m, x, int(i));
            r[i] = ri;
            b0[vox[i]] = float(ri);
            srr = fma(ri, ri, srr);
            sbb = fma(b[i], b[i], sbb);
        }
    }
    const double b1 = block_tree(srr, ws);
    const double b2 = block_tree(sbb, ws);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b1;
        part[nb + blockIdx.x] = b2;
    }
    if (arrive_last(&sc->ticket)) {
        const double rr = final_sum(part, nb, ws);
        const double bb = final_sum(part + nb, nb, ws);
        if (threadIdx.x == 0) {
            sc->rr = rr;
            sc->rr0 = rr;
            sc->bb = bb;
            sc->lim = (tol * tol) * bb;
            sc->k = 0;
            sc->maxit = maxit;
            sc->done = rr <= sc->lim ? 1 : 0;
            sc->converged = sc->done;
            sc->beta = 0.0;
        }
    }
}

// z = double(V-cycle result); partials of r.z and r.z_old; beta.
__global__ void __launch_bounds__(256) mg_gather_kernel(int n, const int* __restrict__ vox,
                                                        const float* __restrict__ xr, const double* __restrict__ r,
                                                        double* __restrict__ z, double* part, MgScalars* sc) {
    if (sc->done) return;
    __shared__ double ws[256];
    const int nb = gridDim.x;
    const int first = sc->k == 0;
    double s0 = 0.0, s1 = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const double zi = double(xr[vox[i]]);
            const double ri = r[i];
            if (!first) s1 = fma(ri, z[i], s1);
            s0 = fma(ri, zi, s0);
            z[i] = zi;
        }
    }
    const double b0 = block_tree(s0, ws);
    const double b1 = block_tree(s1, ws);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b0;
        part[nb + blockIdx.x] = b1;
    }
    if (arrive_last(&sc->ticket)) {
        const double rz = final_sum(part, nb, ws);
        const double rzo = final_sum(part + nb, nb, ws);
        if (threadIdx.x == 0) {
            sc->beta = first ? 0.0 : (rz - rzo) / sc->rz;
            sc->rz = rz;
        }
    }
}

__global__ void __launch_bounds__(256) mg_direction_kernel(int n, const double* __restrict__ z, double* __restrict__ p,
                                                           const MgScalars* sc) {
    if (sc->done) return;
    const long i = long(blockIdx.x) * 256 + threadIdx.x;
    if (i >= n) return;
    p[i] = sc->k == 0 ? z[i] : fma(sc->beta, p[i], z[i]);
}

template <bool Uniform>
__global__ void __launch_bounds__(256) mg_spmv_kernel(DMesh m, const double* __restrict__ p, double* __restrict__ q,
                                                      double* part, MgScalars* sc) {
    if (sc->done) return;
    __shared__ double ws[256];
    const int n = m.n_cells;
    const int nb = gridDim.x;
    double s = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const double qi = apply_M<Uniform>(m, p, int(i));
            q[i] = qi;
            s = fma(p[i], qi, s);
        }
    }
    const double bs = block_tree(s, ws);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (arrive_last(&sc->ticket)) {
        const double pq = final_sum(part, nb, ws);
        if (threadIdx.x == 0) {
            if (pq > 0.0) {
                sc->alpha = sc->rz / pq;
            } else {  // breakdown: the preconditioned direction has no energy
                sc->alpha = 0.0;
                sc->done = 1;
                sc->converged = 0;
            }
        }
    }
}

__global__ void __launch_bounds__(256) mg_axpy_kernel(int n, double* __restrict__ x, double* __restrict__ r,
                                                      const double* __restrict__ p, const double* __restrict__ q,
                                                      const int* __restrict__ vox, float* __restrict__ b0,
                                                      double* part, MgScalars* sc) {
    if (sc->done) return;
    __shared__ double ws[256];
    const int nb = gridDim.x;
    const double alpha = sc->alpha;
    double s = 0.0;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            x[i] = fma(alpha, p[i], x[i]);
            const double ri = fma(-alpha, q[i], r[i]);
            r[i] = ri;
            b0[vox[i]] = float(ri);
            s = fma(ri, ri, s);
        }
    }
    const double bs = block_tree(s, ws);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (arrive_last(&sc->ticket)) {
        const double rr = final_sum(part, nb, ws);
        if (threadIdx.x == 0) {
            const int k = sc->k + 1;
            sc->k = k;
            sc->rr = rr;
            if (rr <= sc->lim) {
                sc->done = 1;
                sc->converged = 1;
            } else if (k >= sc->maxit) {
                sc->done = 1;
                sc->converged = 0;
            }
        }
    }
}

inline int nblk(long n, int bs) { return int((n + bs - 1) / bs); }

// ------------------------------------------------------ host hierarchy ---
struct HostLevel {
    int n[3], cyc[3];
    long V;
    std::vector<double> diag, off;  // off: 6 x V
    std::vector<char> act;
};

long vidx(const HostLevel& L, int i, int j, int k) { return i + long(L.n[0]) * (j + long(L.n[1]) * k); }

// Neighbour voxel of (i, j, k) in direction f; -1 across a non-periodic edge.
long vnbr(const HostLevel& L, int i, int j, int k, int f) {
    int q[3] = {i, j, k};
    const int a = f / 2;
    q[a] += (f & 1) ? 1 : -1;
    if (q[a] < 0 || q[a] >= L.n[a]) {
        if (!L.cyc[a]) return -1;
        q[a] = (q[a] + L.n[a]) % L.n[a];
    }
    return vidx(L, q[0], q[1], q[2]);
}

// Gauss-Jordan inverse with partial pivoting (row-major, in place).
bool invert(std::vector<double>& a, int n) {
    std::vector<double> inv(size_t(n) * n, 0.0);
    for (int i = 0; i < n; ++i) inv[size_t(i) * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[size_t(r) * n + c]) > std::fabs(a[size_t(piv) * n + c])) piv = r;
        if (!(std::fabs(a[size_t(piv) * n + c]) > 0.0)) return false;
        if (piv != c)
            for (int k = 0; k < n; ++k) {
                std::swap(a[size_t(c) * n + k], a[size_t(piv) * n + k]);
                std::swap(inv[size_t(c) * n + k], inv[size_t(piv) * n + k]);
            }
        const double d = 1.0 / a[size_t(c) * n + c];
        for (int k = 0; k < n; ++k) {
            a[size_t(c) * n + k] *= d;
            inv[size_t(c) * n + k] *= d;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = a[size_t(r) * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                a[size_t(r) * n + k] -= f * a[size_t(c) * n + k];
                inv[size_t(r) * n + k] -= f * inv[size_t(c) * n + k];
            }
        }
    }
    a.swap(inv);
    return true;
}

}  // namespace

template <class T>
T* MultigridPCG::dalloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    dev_.push_back(p);
    device_bytes += n * sizeof(T);
    return static_cast<T*>(p);
}

MultigridPCG::~MultigridPCG() {
    if (graph_) cudaGraphExecDestroy(graph_);
    for (void* p : dev_) cudaFree(p);
    if (sc_host_) cudaFreeHost(sc_host_);
}

bool MultigridPCG::init(const pg::HexMesh& m, const std::vector<double>& Mdiag, const std::vector<double>& Moff,
                        const MgSettings& set, std::string* msg) {
    set_ = set;
    set_.pre = std::max(1, std::min(set_.pre, 8));
    set_.post = std::max(0, std::min(set_.post, 8));
    set_.coarsest = std::max(1, std::min(set_.coarsest, 4096));
    const long V0 = long(m.n[0]) * m.n[1] * m.n[2];
    if (V0 <= 0 || long(m.grid_cell.size()) != V0 || long(m.cell_ijk.size()) != 3L * m.n_cells) {
        *msg = "multigrid preconditioner needs a block mesh";
        return false;
    }
    n_cells_ = m.n_cells;
    std::vector<HostLevel> hl(1);
    {
        HostLevel& L = hl[0];
        for (int a = 0; a < 3; ++a) {
            L.n[a] = m.n[a];
            L.cyc[a] = m.cyclic[a];
        }
        L.V = V0;
        L.diag.assign(V0, 1.0);
        L.off.assign(6 * size_t(V0), 0.0);
        L.act.assign(V0, 0);
        for (int c = 0; c < m.n_cells; ++c) {
            const int i = m.cell_ijk[3 * size_t(c)], j = m.cell_ijk[3 * size_t(c) + 1],
                      k = m.cell_ijk[3 * size_t(c) + 2];
            const long v = vidx(L, i, j, k);
            L.diag[v] = Mdiag[c];
            L.act[v] = 1;
            for (int f = 0; f < 6; ++f) {
                const int nb = m.nbr[6 * size_t(c) + f];
                if (nb < 0) continue;
                const long w = vnbr(L, i, j, k, f);
                if (w < 0 || m.grid_cell[w] != nb) {
                    *msg = "multigrid preconditioner: mesh neighbours do not follow the block grid";
                    return false;
                }
                L.off[f * size_t(V0) + v] = Moff[6 * size_t(c) + f];
            }
        }
    }
    // aggregate 2 x 2 x 2 until the level is small enough
    std::vector<std::array<int, 3>> fac;
    while (hl.back().V > set_.coarsest && hl.size() < 16) {
        const HostLevel& F = hl.back();
        std::array<int, 3> fa{};
        HostLevel Cl;
        for (int a = 0; a < 3; ++a) {
            fa[a] = F.n[a] >= 2 ? 2 : 1;
            Cl.n[a] = (F.n[a] + fa[a] - 1) / fa[a];
            Cl.cyc[a] = F.cyc[a];
        }
        Cl.V = long(Cl.n[0]) * Cl.n[1] * Cl.n[2];
        Cl.diag.assign(Cl.V, 0.0);
        Cl.off.assign(6 * size_t(Cl.V), 0.0);
        Cl.act.assign(Cl.V, 0);
        for (int k = 0; k < F.n[2]; ++k)
            for (int j = 0; j < F.n[1]; ++j)
                for (int i = 0; i < F.n[0]; ++i) {
                    const long v = vidx(F, i, j, k);
                    if (!F.act[v]) continue;
                    const int ci = i / fa[0], cj = j / fa[1], ck = k / fa[2];
                    const long I = vidx(Cl, ci, cj, ck);
                    Cl.act[I] = 1;
                    Cl.diag[I] += F.diag[v];
                    for (int f = 0; f < 6; ++f) {
                        const double o = F.off[f * size_t(F.V) + v];
                        if (o == 0.0) continue;
                        int q[3];
                        const long w = vnbr(F, i, j, k, f);
                        if (w < 0) continue;
                        q[0] = int(w % F.n[0]);
                        q[1] = int((w / F.n[0]) % F.n[1]);
                        q[2] = int(w / (long(F.n[0]) * F.n[1]));
                        const long J = vidx(Cl, q[0] / fa[0], q[1] / fa[1], q[2] / fa[2]);
                        if (J == I) {
                            Cl.diag[I] += o;
                        } else {
                            if (vnbr(Cl, ci, cj, ck, f) != J) {
                                *msg = "multigrid preconditioner: aggregate coupling off the grid";
                                return false;
                            }
                            Cl.off[f * size_t(Cl.V) + I] += o;
                        }
                    }
                }
        for (long I = 0; I < Cl.V; ++I)
            if (!Cl.act[I]) Cl.diag[I] = 1.0;
        fac.push_back(fa);
        hl.push_back(std::move(Cl));
    }
    // coarsest level: dense inverse over the active voxels
    const HostLevel& Lc = hl.back();
    std::vector<int> cidx;
    std::vector<long> pos(Lc.V, -1);
    for (long v = 0; v < Lc.V; ++v)
        if (Lc.act[v]) {
            pos[v] = long(cidx.size());
            cidx.push_back(int(v));
        }
    nc_ = int(cidx.size());
    std::vector<double> A(size_t(nc_) * nc_, 0.0);
    double dsum = 0.0;
    for (int r = 0; r < nc_; ++r) {
        const long v = cidx[r];
        const int i = int(v % Lc.n[0]), j = int((v / Lc.n[0]) % Lc.n[1]), k = int(v / (long(Lc.n[0]) * Lc.n[1]));
        A[size_t(r) * nc_ + r] += Lc.diag[v];
        dsum += Lc.diag[v];
        for (int f = 0; f < 6; ++f) {
            const double o = Lc.off[f * size_t(Lc.V) + v];
            if (o == 0.0) continue;
            const long w = vnbr(Lc, i, j, k, f);
            if (w < 0 || pos[w] < 0) continue;
            A[size_t(r) * nc_ + pos[w]] += o;
        }
    }
    if (!m.has_dirichlet && nc_ > 0) {
        // singular (pure Neumann / periodic): invert A + c e e^T, which
        // solves A x = b with e.x = 0 for every b orthogonal to e
        const double c = dsum / (double(nc_) * nc_);
        for (auto& a : A) a += c;
    }
    if (!invert(A, nc_)) {
        *msg = "multigrid preconditioner: singular coarsest operator";
        return false;
    }

    // upload
    lv_.resize(hl.size());
    for (size_t l = 0; l < hl.size(); ++l) {
        const HostLevel& H = hl[l];
        MgLevel& L = lv_[l];
        for (int a = 0; a < 3; ++a) {
            L.n[a] = H.n[a];
            L.cyc[a] = H.cyc[a];
            L.fac[a] = l + 1 < hl.size() ? fac[l][a] : 1;
        }
        L.V = H.V;
        std::vector<float> diag(H.V), inv(H.V), off(6 * size_t(H.V));
        for (long v = 0; v < H.V; ++v) {
            diag[v] = H.act[v] ? float(H.diag[v]) : 1.f;
            inv[v] = H.act[v] ? float(1.0 / H.diag[v]) : 0.f;
        }
        for (size_t e = 0; e < off.size(); ++e) off[e] = float(H.off[e]);
        // uniform: every coupling between two active voxels in direction f
        // has one value; couplings to holes and across edges need none
        L.uniform = 1;
        bool seen[6] = {};
        for (int f = 0; f < 6; ++f) L.coef[f] = 0.f;
        for (int k = 0; k < H.n[2] && L.uniform; ++k)
            for (int j = 0; j < H.n[1] && L.uniform; ++j)
                for (int i = 0; i < H.n[0] && L.uniform; ++i) {
                    const long v = vidx(H, i, j, k);
                    if (!H.act[v]) continue;
                    for (int f = 0; f < 6; ++f) {
                        const long w = vnbr(H, i, j, k, f);
                        if (w < 0 || !H.act[w]) continue;
                        const float o = off[f * size_t(H.V) + v];
                        if (!seen[f]) {
                            seen[f] = true;
                            L.coef[f] = o;
                        } else if (o != L.coef[f]) {
                            L.uniform = 0;
                            break;
                        }
                    }
                }
        if (!(L.diag = dalloc<float>(H.V)) || !(L.inv = dalloc<float>(H.V)) || !(L.b = dalloc<float>(H.V)) ||
            !(L.x = dalloc<float>(H.V)) || !(L.t = dalloc<float>(H.V))) {
            *msg = "multigrid preconditioner: out of device memory";
            return false;
        }
        if (!L.uniform && !(L.off = dalloc<float>(6 * size_t(H.V)))) {
            *msg = "multigrid preconditioner: out of device memory";
            return false;
        }
        cudaMemcpy(L.diag, diag.data(), H.V * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemcpy(L.inv, inv.data(), H.V * sizeof(float), cudaMemcpyHostToDevice);
        if (L.off) cudaMemcpy(L.off, off.data(), off.size() * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemset(L.b, 0, H.V * sizeof(float));
        cudaMemset(L.x, 0, H.V * sizeof(float));
        cudaMemset(L.t, 0, H.V * sizeof(float));
    }
    std::vector<float> cinv(A.begin(), A.end());
    std::vector<int> vox(m.n_cells);
    for (int c = 0; c < m.n_cells; ++c)
        vox[c] = int(vidx(hl[0], m.cell_ijk[3 * size_t(c)], m.cell_ijk[3 * size_t(c) + 1],
                          m.cell_ijk[3 * size_t(c) + 2]));
    const int nb = pcg_blocks(m.n_cells);
    if (!(cidx_ = dalloc<int>(nc_)) || !(cinv_ = dalloc<float>(size_t(nc_) * nc_)) ||
        !(vox_ = dalloc<int>(m.n_cells)) || !(r_ = dalloc<double>(m.n_cells)) || !(z_ = dalloc<double>(m.n_cells)) ||
        !(p_ = dalloc<double>(m.n_cells)) || !(q_ = dalloc<double>(m.n_cells)) ||
        !(part_ = dalloc<double>(2 * size_t(nb) + 8)) || !(sc_ = dalloc<MgScalars>(1))) {
        *msg = "multigrid preconditioner: out of device memory";
        return false;
    }
    cudaMemcpy(cidx_, cidx.data(), nc_ * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(cinv_, cinv.data(), cinv.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(vox_, vox.data(), vox.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemset(sc_, 0, sizeof(MgScalars));
    if (cudaMallocHost(&sc_host_, sizeof(MgScalars)) != cudaSuccess) {
        *msg = "multigrid preconditioner: out of pinned host memory";
        return false;
    }
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        *msg = std::string("multigrid preconditioner: ") + cudaGetErrorString(e);
        return false;
    }
    return true;
}

float* MultigridPCG::result(int l) const {
    if (l == int(lv_.size()) - 1) return lv_[l].x;
    // pre sweeps leave the iterate in x (odd count) or t (even count); the
    // prolongation adds into it; post sweeps alternate from there
    const bool in_x = (set_.pre % 2 == 1) == (set_.post % 2 == 0);
    return in_x ? lv_[l].x : lv_[l].t;
}

int MultigridPCG::vcycle(int l, cudaStream_t s) {
    const MgLevel& L = lv_[l];
    const Lv v = view(L);
    const float om = float(set_.omega);
    if (l == int(lv_.size()) - 1) {
        mg_coarse_kernel<<<nblk(32L * nc_, 256), 256, 0, s>>>(cinv_, cidx_, nc_, L.b, L.x, sc_);
        return 1;
    }
    int launched = 0;
    const int g = nblk(L.V, 256);
    float* cur = L.x;
    float* oth = L.t;
    mg_smooth0_kernel<<<g, 256, 0, s>>>(v, L.b, cur, om, sc_);
    ++launched;
    for (int it = 1; it < set_.pre; ++it) {
        if (L.uniform) mg_smooth_kernel<true><<<g, 256, 0, s>>>(v, L.b, cur, oth, om, sc_);
        else mg_smooth_kernel<false><<<g, 256, 0, s>>>(v, L.b, cur, oth, om, sc_);
        std::swap(cur, oth);
        ++launched;
    }
    const MgLevel& C = lv_[l + 1];
    const Lv cv = view(C);
    if (L.uniform)
        mg_restrict_kernel<true><<<nblk(C.V, 256), 256, 0, s>>>(v, cv, L.fac[0], L.fac[1], L.fac[2], L.b, cur, C.b,
                                                                sc_);
    else
        mg_restrict_kernel<false><<<nblk(C.V, 256), 256, 0, s>>>(v, cv, L.fac[0], L.fac[1], L.fac[2], L.b, cur, C.b,
                                                                 sc_);
    ++launched;
    launched += vcycle(l + 1, s);
    mg_prolong_kernel<<<g, 256, 0, s>>>(v, C.n[0], C.n[1], L.fac[0], L.fac[1], L.fac[2], result(l + 1), cur,
                                        float(set_.scale), sc_);
    ++launched;
    for (int it = 0; it < set_.post; ++it) {
        if (L.uniform) mg_smooth_kernel<true><<<g, 256, 0, s>>>(v, L.b, cur, oth, om, sc_);
        else mg_smooth_kernel<false><<<g, 256, 0, s>>>(v, L.b, cur, oth, om, sc_);
        std::swap(cur, oth);
        ++launched;
    }
    return launched;
}

int MultigridPCG::iteration(const DMesh& dm, double* x, cudaStream_t s) {
    const int n = n_cells_;
    const int nb = pcg_blocks(n);
    int launched = vcycle(0, s);
    mg_gather_kernel<<<nb, 256, 0, s>>>(n, vox_, result(0), r_, z_, part_, sc_);
    mg_direction_kernel<<<nblk(n, 256), 256, 0, s>>>(n, z_, p_, sc_);
    if (dm.lap_uniform) mg_spmv_kernel<true><<<nb, 256, 0, s>>>(dm, p_, q_, part_, sc_);
    else mg_spmv_kernel<false><<<nb, 256, 0, s>>>(dm, p_, q_, part_, sc_);
    mg_axpy_kernel<<<nb, 256, 0, s>>>(n, x, r_, p_, q_, vox_, lv_[0].b, part_, sc_);
    return launched + 4;
}

cudaError_t MultigridPCG::solve(const DMesh& dm, const double* b, double* x, double tol, int maxit,
                                cudaStream_t s, int* iters, double* rr0, double* rr, double* bb, bool* converged) {
    const int n = n_cells_;
    const int nb = pcg_blocks(n);
    if (graph_ && (graph_b_ != b || graph_x_ != x)) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    if (!graph_) {
        cudaGraph_t g;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        graph_launches_ = 0;
        for (int it = 0; it < kGraphIters; ++it) graph_launches_ += iteration(dm, x, s);
        e = cudaStreamEndCapture(s, &g);
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&graph_, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return e;
        graph_b_ = b;
        graph_x_ = x;
    }
    if (dm.lap_uniform) mg_init_kernel<true><<<nb, 256, 0, s>>>(dm, b, x, r_, vox_, lv_[0].b, part_, sc_, tol, maxit);
    else mg_init_kernel<false><<<nb, 256, 0, s>>>(dm, b, x, r_, vox_, lv_[0].b, part_, sc_, tol, maxit);
    ++launches;
    cudaError_t e = cudaMemcpyAsync(sc_host_, sc_, sizeof(MgScalars), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    int replayed = 0;
    while (!sc_host_->done && replayed < maxit) {
        e = cudaGraphLaunch(graph_, s);
        if (e != cudaSuccess) return e;
        replayed += kGraphIters;
        launches += graph_launches_;
        e = cudaMemcpyAsync(sc_host_, sc_, sizeof(MgScalars), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
    }
    *iters = sc_host_->k;
    *rr0 = sc_host_->rr0;
    *rr = sc_host_->rr;
    *bb = sc_host_->bb;
    *converged = sc_host_->converged != 0;
    return cudaGetLastError();
}

}  // namespace pgd
