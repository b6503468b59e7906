// mg.cu -- Poisson solve: FP64 iterative refinement around an FP32
// aggregation-multigrid-preconditioned conjugate gradient (the role of
// OpenFOAM's PCG + GAMG preconditioner for the solve of
// ElectroStaticSolver.C:61-64).
//
// Kernels; every sum runs in a fixed order (no atomics), so a solve is
// bit-reproducible:
//   mg_residual   FP64 r = b - M x over the cells, r.r (and b.b); closes the
//                 outer loop (convergence, power-of-two scale, inner eta)
//   mg_convert    r into the level-0 voxels as FP32 (scaled), d = 0, r.r
//   V-cycle       per level: two Jacobi sweeps from the zero guess in one
//                 pass, residual + restriction to the aggregates, coarse
//                 level, prolongation, Jacobi sweeps; the last level-0 sweep
//                 also forms r.z and beta; dense inverse times vector on the
//                 coarsest level
//   mg_spmv       p = z + beta p (formed at the stencil points) and q = A p
//                 in one pass, p.q and q.z -> alpha
//   mg_axpy       d += alpha p, r -= alpha q, r.r; closes the inner loop
//   mg_update     FP64 x += d / scale
// Voxel kernels run on 3-D grids (x-y tiles, one grid slice per plane), so a
// thread's (i, j, k) come without a division.
#include "mg.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "fields.h"
#include "reduce.cuh"

namespace pgd {

namespace {

constexpr int kInnerMax = 200;     // inner iterations per outer step
constexpr int kOuterMax = 64;      // outer steps per solve
constexpr double kEtaMin = 1e-4;   // deepest relative reduction asked of one FP32 inner solve

// Level description passed by value to the FP32 kernels (32-bit indices:
// a level holds fewer than 2^31 voxels).
struct Lv {
    int X, Y, Z, cx, cy, cz;
    int V;
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
    v.V = int(L.V);
    v.uniform = L.uniform;
    for (int f = 0; f < 6; ++f) v.coef[f] = L.coef[f];
    v.diag = L.diag;
    v.inv = L.inv;
    v.off = L.off;
    return v;
}

// Launch shape of a voxel kernel: 256-thread blocks tiling an x-y plane as
// BX x BY, one grid z-slice per plane, so that a thread's (i, j, k) come
// from its indices without a division.
struct Shape {
    dim3 grid, block;
    int blocks;
};

int pow2_at_least(int n, int cap) {
    int p = 1;
    while (p < n && p < cap) p <<= 1;
    return p;
}

// Rows of up to 32 x-neighbours; thin planes (small Y) get wider x-tiles so
// that few threads fall outside the grid.
Shape shape(int X, int Y, int Z) {
    const int by = std::min(256 / pow2_at_least(X, 32), pow2_at_least(Y, 256));
    const int bx = 256 / by;
    Shape s;
    s.block = dim3(bx, by, 1);
    s.grid = dim3((X + bx - 1) / bx, (Y + by - 1) / by, Z);
    s.blocks = int(s.grid.x * s.grid.y * s.grid.z);
    return s;
}

Shape shape(const MgLevel& L) { return shape(L.n[0], L.n[1], L.n[2]); }

// The level-0 kernels that end in a grid-wide sum give each thread kZB
// z-planes, so that the last block combines kZB times fewer partials.
constexpr int kZB = 4;

Shape shape_sum(const MgLevel& L) {
    Shape s = shape(L);
    s.grid.z = (L.n[2] + kZB - 1) / kZB;
    s.blocks = int(s.grid.x * s.grid.y * s.grid.z);
    return s;
}

__device__ __forceinline__ bool coords(const Lv& L, int& i, int& j, int& k, int& v) {
    i = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    k = blockIdx.z;
    v = i + L.X * (j + L.Y * k);
    return i < L.X && j < L.Y;
}

// Plane kz of the kZB planes of a shape_sum block.
__device__ __forceinline__ bool coords_sum(const Lv& L, int kz, int& i, int& j, int& k, int& v) {
    i = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    k = blockIdx.z * kZB + kz;
    v = i + L.X * (j + L.Y * k);
    return i < L.X && j < L.Y && k < L.Z;
}

// (A u)_v on one level for a field given by val(w).  A neighbour across a
// non-periodic edge has no coupling (its coefficient is zero, the index falls
// back to v itself); a hole neighbour holds zero, so the uniform form may use
// coef[f] there.
template <bool Uniform, class Val>
__device__ __forceinline__ float apply_A(const Lv& L, int i, int j, int k, int v, Val val) {
    const int X = L.X, XY = L.X * L.Y;
    int nb[6];
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
    float s = L.diag[v] * val(v);
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const float a = Uniform ? (ok[f] ? L.coef[f] : 0.f) : L.off[f * L.V + v];
        s = fmaf(a, val(nb[f]), s);
    }
    return s;
}

// ------------------------------------------------------------ V-cycle ----
// One sweep from a zero guess: y = omega D^-1 b.
__global__ void __launch_bounds__(256) mg_smooth0_kernel(Lv L, const float* __restrict__ b, float* __restrict__ y,
                                                         float omega) {
    int i, j, k, v;
    if (!coords(L, i, j, k, v)) return;
    y[v] = (omega * L.inv[v]) * b[v];
}

// Two sweeps from a zero guess in one pass: x1 = omega D^-1 b is formed on
// the fly at the seven stencil points, y = x1 + omega D^-1 (b - A x1).
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_smooth01_kernel(Lv L, const float* __restrict__ b, float* __restrict__ y,
                                                          float omega) {
    int i, j, k, v;
    if (!coords(L, i, j, k, v)) return;
    const float* __restrict__ inv = L.inv;
    auto x1 = [&](int w) { return (omega * inv[w]) * b[w]; };
    const float ax = apply_A<Uniform>(L, i, j, k, v, x1);
    y[v] = fmaf(omega * inv[v], b[v] - ax, x1(v));
}

// One weighted-Jacobi sweep: y = x + omega D^-1 (b - A x).
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_smooth_kernel(Lv L, const float* __restrict__ b,
                                                        const float* __restrict__ x, float* __restrict__ y,
                                                        float omega) {
    int i, j, k, v;
    if (!coords(L, i, j, k, v)) return;
    const float ax = apply_A<Uniform>(L, i, j, k, v, [&](int w) { return x[w]; });
    y[v] = fmaf(omega * L.inv[v], b[v] - ax, x[v]);
}

// Closes the preconditioner application: rz = r.z, and the flexible
// (Polak-Ribiere) beta = (r.z - r.z_old) / rz_old with
// r.z_old = rz_old - alpha q.z_old from the previous iteration.
__device__ __forceinline__ void finish_rz(float prod, float* wsf, double* ws, double* part, MgScalars* sc) {
    const float bs = block_tree_f(prod, wsf);
    if (flat_tid() == 0) part[flat_bid()] = double(bs);
    if (arrive_last(&sc->ticket)) {
        const double rz = final_sum(part, int(grid_blocks()), ws);
        if (flat_tid() == 0) {
            const double rzo = sc->rz - sc->alpha * sc->qz;
            sc->beta = sc->k == 0 ? 0.0 : (rz - rzo) / sc->rz;
            sc->rz = rz;
        }
    }
}

// The last level-0 sweep, which also forms r.z (b is the inner residual r).
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_smooth_dot_kernel(Lv L, const float* __restrict__ b,
                                                            const float* __restrict__ x, float* __restrict__ y,
                                                            float omega, double* part, MgScalars* sc) {
    __shared__ float wsf[256];
    __shared__ double ws[256];
    float prod = 0.f;
#pragma unroll
    for (int kz = 0; kz < kZB; ++kz) {
        int i, j, k, v;
        if (!coords_sum(L, kz, i, j, k, v)) continue;
        const float ax = apply_A<Uniform>(L, i, j, k, v, [&](int w) { return x[w]; });
        const float bv = b[v];
        const float yv = fmaf(omega * L.inv[v], bv - ax, x[v]);
        y[v] = yv;
        prod = fmaf(bv, yv, prod);
    }
    finish_rz(prod, wsf, ws, part, sc);
}

// r.z alone (no post sweeps, or a single-level hierarchy).
__global__ void __launch_bounds__(256) mg_rz_kernel(Lv L, const float* __restrict__ r, const float* __restrict__ z,
                                                    double* part, MgScalars* sc) {
    __shared__ float wsf[256];
    __shared__ double ws[256];
    float prod = 0.f;
#pragma unroll
    for (int kz = 0; kz < kZB; ++kz) {
        int i, j, k, v;
        if (coords_sum(L, kz, i, j, k, v)) prod = fmaf(r[v], z[v], prod);
    }
    finish_rz(prod, wsf, ws, part, sc);
}

// Coarse right-hand side: bc[I] = sum over the active children of I of
// (b - A x), children in x-fastest order; sx, sy, sz are the aggregation
// shifts (1: pairs, 0: none) of each axis.
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_restrict_kernel(Lv F, Lv Cl, int sx, int sy, int sz,
                                                          const float* __restrict__ b, const float* __restrict__ x,
                                                          float* __restrict__ bc) {
    int ci, cj, ck, I;
    if (!coords(Cl, ci, cj, ck, I)) return;
    auto xv = [&](int w) { return x[w]; };
    float s = 0.f;
#pragma unroll
    for (int dz = 0; dz < 2; ++dz) {
        const int k = (ck << sz) + dz;
        if (dz > sz || k >= F.Z) continue;
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const int j = (cj << sy) + dy;
            if (dy > sy || j >= F.Y) continue;
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                const int i = (ci << sx) + dx;
                if (dx > sx || i >= F.X) continue;
                const int v = i + F.X * (j + F.Y * k);
                if (F.inv[v] != 0.f) s += b[v] - apply_A<Uniform>(F, i, j, k, v, xv);
            }
        }
    }
    bc[I] = s;
}

// x += scale * xc[parent] on the active voxels.
__global__ void __launch_bounds__(256) mg_prolong_kernel(Lv F, int CX, int CY, int sx, int sy, int sz,
                                                         const float* __restrict__ xc, float* __restrict__ x,
                                                         float scale) {
    int i, j, k, v;
    if (!coords(F, i, j, k, v)) return;
    if (F.inv[v] == 0.f) return;
    const int I = (i >> sx) + CX * ((j >> sy) + CY * (k >> sz));
    x[v] = fmaf(scale, xc[I], x[v]);
}

// The prolongation fused into the first post sweep: x' = x + scale xc[parent]
// on the active voxels (zero on holes), formed at the seven stencil points
// from their own (i, j, k), then y = x' + omega D^-1 (b - A x').
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_prolong_smooth_kernel(Lv L, int CX, int CY, int sx, int sy, int sz,
                                                                const float* __restrict__ xc,
                                                                const float* __restrict__ b,
                                                                const float* __restrict__ x, float* __restrict__ y,
                                                                float scale, float omega) {
    int i, j, k, v;
    if (!coords(L, i, j, k, v)) return;
    const int X = L.X, XY = L.X * L.Y;
    auto xp = [&](int w, int wi, int wj, int wk) {
        if (L.inv[w] == 0.f) return 0.f;
        return fmaf(scale, xc[(wi >> sx) + CX * ((wj >> sy) + CY * (wk >> sz))], x[w]);
    };
    // neighbours: index and coordinates, with the periodic wrap; across a
    // non-periodic edge the point is v itself with a zero coefficient
    int ni[6], nj[6], nk[6], nb[6];
    bool ok[6];
    ok[0] = i > 0 || L.cx;
    ni[0] = i > 0 ? i - 1 : (L.cx ? L.X - 1 : i);
    ok[1] = i < L.X - 1 || L.cx;
    ni[1] = i < L.X - 1 ? i + 1 : (L.cx ? 0 : i);
    nj[0] = nj[1] = j;
    nk[0] = nk[1] = k;
    ok[2] = j > 0 || L.cy;
    nj[2] = j > 0 ? j - 1 : (L.cy ? L.Y - 1 : j);
    ok[3] = j < L.Y - 1 || L.cy;
    nj[3] = j < L.Y - 1 ? j + 1 : (L.cy ? 0 : j);
    ni[2] = ni[3] = i;
    nk[2] = nk[3] = k;
    ok[4] = k > 0 || L.cz;
    nk[4] = k > 0 ? k - 1 : (L.cz ? L.Z - 1 : k);
    ok[5] = k < L.Z - 1 || L.cz;
    nk[5] = k < L.Z - 1 ? k + 1 : (L.cz ? 0 : k);
    ni[4] = ni[5] = i;
    nj[4] = nj[5] = j;
    for (int f = 0; f < 6; ++f) nb[f] = ni[f] + X * nj[f] + XY * nk[f];
    const float xv = xp(v, i, j, k);
    float s = L.diag[v] * xv;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const float a = Uniform ? (ok[f] ? L.coef[f] : 0.f) : L.off[f * L.V + v];
        s = fmaf(a, xp(nb[f], ni[f], nj[f], nk[f]), s);
    }
    y[v] = fmaf(omega * L.inv[v], b[v] - s, xv);
}

// Coarsest level: x[idx[r]] = sum_k inv[r][k] b[idx[k]], one warp per row,
// lane l adds k = l, l + 32, ... then an xor-tree.
__global__ void __launch_bounds__(256) mg_coarse_kernel(const float* __restrict__ inv, const int* __restrict__ idx,
                                                        int nc, const float* __restrict__ b, float* __restrict__ x) {
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

// ------------------------------------------------------- FP32 inner PCG --
// New direction and its image in one pass: p = z + beta p_old is formed at
// the seven stencil points, q = A p on the active voxels (0 on holes); p.q
// and q.z -> alpha.  p alternates between two buffers by iteration parity
// (p_old = pb[k & 1], p = pb[(k + 1) & 1]), so a fixed kernel sequence serves
// every iteration.
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_spmv_kernel(Lv L, const float* __restrict__ z, float* __restrict__ pb,
                                                      float* __restrict__ q, double* part, MgScalars* sc) {
    __shared__ float wsf[256];
    __shared__ double ws[256];
    const int it = sc->k;
    const float beta = it == 0 ? 0.f : float(sc->beta);
    const float* __restrict__ pold = pb + size_t(it & 1) * L.V;
    float* __restrict__ pnew = pb + size_t((it + 1) & 1) * L.V;
    auto pv = [&](int u) { return fmaf(beta, pold[u], z[u]); };
    float spq = 0.f, sqz = 0.f;
#pragma unroll
    for (int kz = 0; kz < kZB; ++kz) {
        int i, j, k, v;
        if (!coords_sum(L, kz, i, j, k, v)) continue;
        const float pc = pv(v);
        float qv = 0.f;
        if (L.inv[v] != 0.f) qv = apply_A<Uniform>(L, i, j, k, v, pv);
        pnew[v] = pc;
        q[v] = qv;
        spq = fmaf(pc, qv, spq);
        sqz = fmaf(qv, z[v], sqz);
    }
    const float b0 = block_tree_f(spq, wsf);
    const float b1 = block_tree_f(sqz, wsf);
    const int nb = int(grid_blocks());
    if (flat_tid() == 0) {
        part[flat_bid()] = double(b0);
        part[nb + flat_bid()] = double(b1);
    }
    if (arrive_last(&sc->ticket)) {
        const double pq = final_sum(part, nb, ws);
        const double qz = final_sum(part + nb, nb, ws);
        if (flat_tid() == 0) {
            sc->qz = qz;
            if (pq > 0.0 && sc->rz > 0.0) {
                sc->alpha = sc->rz / pq;
            } else {  // breakdown: the direction carries no energy
                sc->alpha = 0.0;
                sc->idone = 1;
            }
        }
    }
}

// d += alpha p, r -= alpha q, r.r; ends the inner loop on convergence or at
// the iteration caps (graph: through the loop's condition).
__global__ void __launch_bounds__(256) mg_axpy_kernel(Lv L, float* __restrict__ d, float* __restrict__ r,
                                                      const float* __restrict__ pb, const float* __restrict__ q,
                                                      double* part, MgScalars* sc, unsigned int* guard,
                                                      int maxit, cudaGraphConditionalHandle inner, int graph) {
    __shared__ float wsf[256];
    __shared__ double ws[256];
    const float alpha = float(sc->alpha);
    const float* __restrict__ p = pb + size_t((sc->k + 1) & 1) * L.V;
    float srr = 0.f;
#pragma unroll
    for (int kz = 0; kz < kZB; ++kz) {
        int i, j, k, v;
        if (!coords_sum(L, kz, i, j, k, v)) continue;
        d[v] = fmaf(alpha, p[v], d[v]);
        const float rv = fmaf(-alpha, q[v], r[v]);
        r[v] = rv;
        srr = fmaf(rv, rv, srr);
    }
    const float bs = block_tree_f(srr, wsf);
    if (flat_tid() == 0) part[flat_bid()] = double(bs);
    if (arrive_last(&sc->ticket)) {
        const double rr = final_sum(part, int(grid_blocks()), ws);
        if (flat_tid() == 0) {
            const int kk = sc->k + 1;
            const int total = sc->total + 1;
            const unsigned int g = *guard + 1u;
            *guard = g;
            sc->k = kk;
            sc->total = total;
            sc->irr = rr;
            // caps written so that out-of-range counters also end the loop
            const int done = sc->idone || !(rr > sc->ilim) || !(kk > 0 && kk < kInnerMax) ||
                             !(total > 0 && total < maxit) || g >= unsigned(maxit);
            sc->idone = done;
            if (graph) cudaGraphSetConditional(inner, done ? 0u : 1u);
        }
    }
}

// ------------------------------------------------------- FP64 outer loop --
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

// r = b - M x; r.r (first: and b.b).  The last block closes the outer loop:
// converged when ||r||2 <= tol ||b||2; otherwise the next inner solve gets
// the power-of-two scale that brings r to unit RMS and the relative
// reduction eta it needs (clamped to [kEtaMin, 0.5]).
template <bool Uniform>
__global__ void __launch_bounds__(256) mg_residual_kernel(DMesh m, const double* __restrict__ b,
                                                          const double* __restrict__ x, double* __restrict__ r,
                                                          double* part, MgScalars* sc, int first, double tol,
                                                          int maxit, unsigned int* guard,
                                                          cudaGraphConditionalHandle outer, int graph) {
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
            srr = fma(ri, ri, srr);
            if (first) sbb = fma(b[i], b[i], sbb);
        }
    }
    const double b1 = block_tree(srr, ws);
    const double b2 = first ? block_tree(sbb, ws) : 0.0;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b1;
        part[nb + blockIdx.x] = b2;
    }
    if (arrive_last(&sc->ticket)) {
        const double rr = final_sum(part, nb, ws);
        const double bb = first ? final_sum(part + nb, nb, ws) : 0.0;
        if (threadIdx.x == 0) {
            if (first) {
                sc->bb = bb;
                sc->lim = (tol * tol) * bb;
                sc->rr0 = rr;
                sc->total = 0;
                sc->outer = 0;
                sc->maxit = maxit;
                sc->rz = 0.0;
                sc->alpha = 0.0;
                sc->qz = 0.0;
            } else {
                sc->outer = sc->outer + 1;
            }
            sc->rr = rr;
            const int conv = !(rr > sc->lim);
            if (first) *guard = 0u;
            const int t = sc->total, o = sc->outer;
            const int done = conv || !(t >= 0 && t < maxit) || !(o >= 0 && o < kOuterMax) || !(rr == rr) ||
                             *guard >= unsigned(maxit);
            sc->converged = conv;
            sc->done = done;
            double scale = 1.0;
            if (rr > 0.0) scale = ldexp(1.0, -ilogb(sqrt(rr / double(n))));
            sc->scale = scale;
            sc->inv_scale = 1.0 / scale;
            const double need = rr > 0.0 ? 0.5 * sqrt(sc->lim / rr) : 1.0;
            sc->eta = fmin(fmax(need, kEtaMin), 0.5);
            if (graph) cudaGraphSetConditional(outer, done ? 0u : 1u);
        }
    }
}

// Level-0 inner residual r32 = scale * r (cells -> voxels), d = 0; r.r
// starts the inner loop.
__global__ void __launch_bounds__(256) mg_convert_kernel(int n, const int* __restrict__ vox,
                                                         const double* __restrict__ r, float* __restrict__ r32,
                                                         float* __restrict__ d, double* part, MgScalars* sc,
                                                         int maxit, cudaGraphConditionalHandle inner, int graph) {
    __shared__ float wsf[256];
    __shared__ double ws[256];
    const double scale = sc->scale;
    float srr = 0.f;
    const long base = long(blockIdx.x) * kChunk + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const long i = base + j * 256;
        if (i < n) {
            const int v = vox[i];
            const float rv = float(r[i] * scale);
            r32[v] = rv;
            d[v] = 0.f;
            srr = fmaf(rv, rv, srr);
        }
    }
    const float bs = block_tree_f(srr, wsf);
    if (threadIdx.x == 0) part[blockIdx.x] = double(bs);
    if (arrive_last(&sc->ticket)) {
        const double rr = final_sum(part, gridDim.x, ws);
        if (threadIdx.x == 0) {
            sc->irr = rr;
            sc->ilim = sc->eta * sc->eta * rr;
            sc->k = 0;
            const int t = sc->total;
            const int done = !(rr > 0.0) || !(t >= 0 && t < maxit);
            sc->idone = done;
            if (graph) cudaGraphSetConditional(inner, done ? 0u : 1u);
        }
    }
}

// x += d / scale (FP64).
__global__ void __launch_bounds__(256) mg_update_kernel(int n, const int* __restrict__ vox,
                                                        const float* __restrict__ d, double* __restrict__ x,
                                                        const MgScalars* sc) {
    const long i = long(blockIdx.x) * 256 + threadIdx.x;
    if (i >= n) return;
    x[i] = fma(double(d[vox[i]]), sc->inv_scale, x[i]);
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
    if (exec_) cudaGraphExecDestroy(exec_);
    for (void* p : dev_) cudaFree(p);
    if (sc_host_) cudaFreeHost(sc_host_);
}

bool MultigridPCG::init(const pg::HexMesh& m, const std::vector<double>& Mdiag, const std::vector<double>& Moff,
                        const MgSettings& set, std::string* msg) {
    set_ = set;
    const char* g = std::getenv("PICGPU_MG_GRAPH");
    use_graph_ = !(g && g[0] == '0');
    set_.pre = std::max(1, std::min(set_.pre, 8));
    set_.post = std::max(0, std::min(set_.post, 8));
    set_.coarsest = std::max(1, std::min(set_.coarsest, 4096));
    const long G0 = long(m.n[0]) * m.n[1] * m.n[2];
    if (G0 >= (1L << 31) || m.n[2] > 65535) {
        *msg = "multigrid preconditioner: at most 2^31 block cells and 65535 cells along z";
        return false;
    }
    if (G0 <= 0 || long(m.grid_cell.size()) != G0 || long(m.cell_ijk.size()) != 3L * m.n_cells) {
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
        L.V = G0;
        L.diag.assign(G0, 1.0);
        L.off.assign(6 * size_t(G0), 0.0);
        L.act.assign(G0, 0);
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
                L.off[f * size_t(G0) + v] = Moff[6 * size_t(c) + f];
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
    const long V0 = hl[0].V;
    // block partials: the widest reduction launch (cells, or the level-0 grid)
    const long nbmax = std::max<long>(pcg_blocks(m.n_cells), shape(lv_[0]).blocks);
    part_cap_ = 2 * nbmax + 8;
    if (!(cidx_ = dalloc<int>(nc_)) || !(cinv_ = dalloc<float>(size_t(nc_) * nc_)) ||
        !(vox_ = dalloc<int>(m.n_cells)) || !(r64_ = dalloc<double>(m.n_cells)) || !(d_ = dalloc<float>(V0)) ||
        !(p_ = dalloc<float>(2 * V0)) || !(q_ = dalloc<float>(V0)) || !(part_ = dalloc<double>(size_t(part_cap_))) ||
        !(sc_ = dalloc<MgScalars>(1)) || !(guard_ = dalloc<unsigned int>(1))) {
        *msg = "multigrid preconditioner: out of device memory";
        return false;
    }
    cudaMemset(d_, 0, V0 * sizeof(float));
    cudaMemset(p_, 0, 2 * V0 * sizeof(float));
    cudaMemset(q_, 0, V0 * sizeof(float));
    cudaMemcpy(cidx_, cidx.data(), nc_ * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(cinv_, cinv.data(), cinv.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(vox_, vox.data(), vox.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemset(sc_, 0, sizeof(MgScalars));
    cudaMemset(guard_, 0, sizeof(unsigned int));
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
    // the pre sweeps leave the iterate in x: a lone zero-guess sweep or the
    // fused two-sweep kernel write x, each further sweep swaps x and t; the
    // prolongation adds into it and each post sweep swaps again
    const int swaps = std::max(0, set_.pre - 2) + set_.post;
    return swaps % 2 == 0 ? lv_[l].x : lv_[l].t;
}

int MultigridPCG::vcycle(int l, cudaStream_t s) {
    const MgLevel& L = lv_[l];
    const Lv v = view(L);
    const Shape sh = shape(L);
    const float om = float(set_.omega);
    if (l == int(lv_.size()) - 1) {
        mg_coarse_kernel<<<nblk(32L * nc_, 256), 256, 0, s>>>(cinv_, cidx_, nc_, L.b, L.x);
        if (l > 0) return 1;
        const Shape ss = shape_sum(L);
        mg_rz_kernel<<<ss.grid, ss.block, 0, s>>>(v, L.b, L.x, part_, sc_);
        return 2;
    }
    int launched = 0;
    float* cur = L.x;
    float* oth = L.t;
    if (set_.pre == 1) {
        mg_smooth0_kernel<<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, om);
    } else {
        if (L.uniform) mg_smooth01_kernel<true><<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, om);
        else mg_smooth01_kernel<false><<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, om);
    }
    ++launched;
    for (int it = 2; it < set_.pre; ++it) {
        if (L.uniform) mg_smooth_kernel<true><<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, oth, om);
        else mg_smooth_kernel<false><<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, oth, om);
        std::swap(cur, oth);
        ++launched;
    }
    const MgLevel& C = lv_[l + 1];
    const Lv cv = view(C);
    const Shape cs = shape(C);
    const int sx = L.fac[0] - 1, sy = L.fac[1] - 1, sz = L.fac[2] - 1;
    if (L.uniform)
        mg_restrict_kernel<true><<<cs.grid, cs.block, 0, s>>>(v, cv, sx, sy, sz, L.b, cur, C.b);
    else
        mg_restrict_kernel<false><<<cs.grid, cs.block, 0, s>>>(v, cv, sx, sy, sz, L.b, cur, C.b);
    ++launched;
    launched += vcycle(l + 1, s);
    const bool fuse = set_.post >= 1 && !(l == 0 && set_.post == 1);
    if (fuse) {
        // the prolongation inside the first post sweep
        if (L.uniform)
            mg_prolong_smooth_kernel<true><<<sh.grid, sh.block, 0, s>>>(v, C.n[0], C.n[1], sx, sy, sz, result(l + 1),
                                                                        L.b, cur, oth, float(set_.scale), om);
        else
            mg_prolong_smooth_kernel<false><<<sh.grid, sh.block, 0, s>>>(v, C.n[0], C.n[1], sx, sy, sz,
                                                                         result(l + 1), L.b, cur, oth,
                                                                         float(set_.scale), om);
        std::swap(cur, oth);
    } else {
        mg_prolong_kernel<<<sh.grid, sh.block, 0, s>>>(v, C.n[0], C.n[1], sx, sy, sz, result(l + 1), cur,
                                                      float(set_.scale));
    }
    ++launched;
    for (int it = fuse ? 1 : 0; it < set_.post; ++it) {
        const bool last0 = l == 0 && it == set_.post - 1;
        if (last0) {
            const Shape ss = shape_sum(L);
            if (L.uniform) mg_smooth_dot_kernel<true><<<ss.grid, ss.block, 0, s>>>(v, L.b, cur, oth, om, part_, sc_);
            else mg_smooth_dot_kernel<false><<<ss.grid, ss.block, 0, s>>>(v, L.b, cur, oth, om, part_, sc_);
        } else {
            if (L.uniform) mg_smooth_kernel<true><<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, oth, om);
            else mg_smooth_kernel<false><<<sh.grid, sh.block, 0, s>>>(v, L.b, cur, oth, om);
        }
        std::swap(cur, oth);
        ++launched;
    }
    if (l == 0 && set_.post == 0) {
        const Shape ss = shape_sum(L);
        mg_rz_kernel<<<ss.grid, ss.block, 0, s>>>(v, L.b, cur, part_, sc_);
        ++launched;
    }
    return launched;
}

// One inner iteration: V-cycle (ends with r.z and beta), direction + A p,
// update of d and r.
int MultigridPCG::inner_iteration(cudaStream_t s, int maxit, cudaGraphConditionalHandle h_inner, int graph) {
    const MgLevel& L0 = lv_[0];
    const Lv v0 = view(L0);
    const Shape sh = shape_sum(L0);
    int launched = vcycle(0, s);
    float* z = result(0);
    if (L0.uniform) mg_spmv_kernel<true><<<sh.grid, sh.block, 0, s>>>(v0, z, p_, q_, part_, sc_);
    else mg_spmv_kernel<false><<<sh.grid, sh.block, 0, s>>>(v0, z, p_, q_, part_, sc_);
    mg_axpy_kernel<<<sh.grid, sh.block, 0, s>>>(v0, d_, L0.b, p_, q_, part_, sc_, guard_, maxit, h_inner, graph);
    return launched + 2;
}

void MultigridPCG::residual(const DMesh& dm, const double* b, double* x, int first, double tol, int maxit,
                            cudaStream_t s, cudaGraphConditionalHandle h_outer, int graph) {
    const int nbc = pcg_blocks(n_cells_);
    if (dm.lap_uniform)
        mg_residual_kernel<true><<<nbc, 256, 0, s>>>(dm, b, x, r64_, part_, sc_, first, tol, maxit, guard_, h_outer,
                                                      graph);
    else
        mg_residual_kernel<false><<<nbc, 256, 0, s>>>(dm, b, x, r64_, part_, sc_, first, tol, maxit, guard_, h_outer,
                                                       graph);
}

// The solve graph:
//   residual(first) -> while (outer) { convert -> while (inner) { V-cycle,
//   direction + A p, axpy } -> update -> residual }
cudaError_t MultigridPCG::build_graph(const DMesh& dm, const double* b, double* x, double tol, int maxit,
                                      cudaStream_t s) {
    if (exec_) {
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
    }
    const int n = n_cells_;
    const int nbc = pcg_blocks(n);
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaGraph_t main = nullptr;
    cudaError_t e = cudaGraphCreate(&main, 0);
    if (e != cudaSuccess) return e;
    auto fail = [&](cudaError_t err) {
        cudaGraphDestroy(main);
        return err;
    };
    cudaGraphConditionalHandle h_outer, h_inner;
    if ((e = cudaGraphConditionalHandleCreate(&h_outer, main, 0, cudaGraphCondAssignDefault))) return fail(e);
    // captured kernels go into `g` after `deps`; `tail` receives the last nodes
    auto capture = [&](cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, auto&& body,
                       std::vector<cudaGraphNode_t>* tail) -> cudaError_t {
        cudaError_t err = cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                                        deps.size(), mode);
        if (err != cudaSuccess) return err;
        body();
        if (tail) {
            cudaStreamCaptureStatus st;
            const cudaGraphNode_t* d = nullptr;
            size_t nd = 0;
            err = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &d, nullptr, &nd);
            if (err == cudaSuccess) tail->assign(d, d + nd);
        }
        cudaGraph_t out = g;
        const cudaError_t err2 = cudaStreamEndCapture(s, &out);
        return err != cudaSuccess ? err : err2;
    };
    auto add_while = [&](cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle h,
                         cudaGraphNode_t* node, cudaGraph_t* body) -> cudaError_t {
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        const cudaError_t err = cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                                 deps.size(), &np);
        if (err == cudaSuccess) *body = np.conditional.phGraph_out[0];
        return err;
    };
    std::vector<cudaGraphNode_t> tail;
    e = capture(main, {}, [&] { residual(dm, b, x, 1, tol, maxit, s, h_outer, 1); }, &tail);
    if (e) return fail(e);
    cudaGraphNode_t w_outer, w_inner;
    cudaGraph_t body_outer, body_inner;
    if ((e = add_while(main, tail, h_outer, &w_outer, &body_outer))) return fail(e);
    if ((e = cudaGraphConditionalHandleCreate(&h_inner, body_outer, 0, cudaGraphCondAssignDefault))) return fail(e);
    e = capture(body_outer, {}, [&] {
        mg_convert_kernel<<<nbc, 256, 0, s>>>(n, vox_, r64_, lv_[0].b, d_, part_, sc_, maxit, h_inner, 1);
    }, &tail);
    if (e) return fail(e);
    if ((e = add_while(body_outer, tail, h_inner, &w_inner, &body_inner))) return fail(e);
    int inner = 0;
    e = capture(body_inner, {}, [&] { inner = inner_iteration(s, maxit, h_inner, 1); }, nullptr);
    if (e) return fail(e);
    e = capture(body_outer, {w_inner}, [&] {
        mg_update_kernel<<<nblk(n, 256), 256, 0, s>>>(n, vox_, d_, x, sc_);
        residual(dm, b, x, 0, tol, maxit, s, h_outer, 1);
    }, nullptr);
    if (e) return fail(e);
    e = cudaGraphInstantiate(&exec_, main, 0);
    cudaGraphDestroy(main);
    if (e != cudaSuccess) return e;
    inner_launches_ = inner;
    outer_launches_ = 3;
    graph_b_ = b;
    graph_x_ = x;
    graph_tol_ = tol;
    graph_maxit_ = maxit;
    return cudaSuccess;
}

// The same kernel sequence driven from the host, which reads the loop flags
// after each closing kernel (used when graphs are switched off, e.g. for
// kernel profilers that cannot see into conditional graph nodes).
cudaError_t MultigridPCG::solve_eager(const DMesh& dm, const double* b, double* x, double tol, int maxit,
                                      cudaStream_t s) {
    const int n = n_cells_;
    const int nbc = pcg_blocks(n);
    auto read = [&]() {
        cudaError_t e = cudaMemcpyAsync(sc_host_, sc_, sizeof(MgScalars), cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    };
    cudaError_t e;
    residual(dm, b, x, 1, tol, maxit, s, 0, 0);
    launches += 1;
    if ((e = read())) return e;
    while (!sc_host_->done) {
        mg_convert_kernel<<<nbc, 256, 0, s>>>(n, vox_, r64_, lv_[0].b, d_, part_, sc_, maxit, 0, 0);
        launches += 1;
        if ((e = read())) return e;
        while (!sc_host_->idone) {
            launches += inner_iteration(s, maxit, 0, 0);
            if ((e = read())) return e;
        }
        mg_update_kernel<<<nblk(n, 256), 256, 0, s>>>(n, vox_, d_, x, sc_);
        residual(dm, b, x, 0, tol, maxit, s, 0, 0);
        launches += 2;
        if ((e = read())) return e;
    }
    return cudaGetLastError();
}

cudaError_t MultigridPCG::solve(const DMesh& dm, const double* b, double* x, double tol, int maxit, cudaStream_t s,
                                int* iters, int* outer, double* rr0, double* rr, double* bb, bool* converged) {
    cudaError_t e;
    // every reduction launch must fit the partials buffer
    if (2L * std::max<long>(pcg_blocks(n_cells_), shape(lv_[0]).blocks) + 8 > part_cap_ || maxit < 1)
        return cudaErrorInvalidValue;
    if (use_graph_) {
        if (!exec_ || graph_b_ != b || graph_x_ != x || graph_tol_ != tol || graph_maxit_ != maxit)
            if ((e = build_graph(dm, b, x, tol, maxit, s)) != cudaSuccess) return e;
        if ((e = cudaGraphLaunch(exec_, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(sc_host_, sc_, sizeof(MgScalars), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        launches += 1 + int64_t(sc_host_->outer) * outer_launches_ + int64_t(sc_host_->total) * inner_launches_;
    } else if ((e = solve_eager(dm, b, x, tol, maxit, s)) != cudaSuccess) {
        return e;
    }
    *iters = sc_host_->total;
    *outer = sc_host_->outer;
    *rr0 = sc_host_->rr0;
    *rr = sc_host_->rr;
    *bb = sc_host_->bb;
    *converged = sc_host_->converged != 0;
    return cudaGetLastError();
}

}  // namespace pgd
