// mg.h -- Poisson solve by FP64 iterative refinement around an FP32
// multigrid-preconditioned conjugate gradient.
//
// The Poisson operator M (SPD, -laplacian) of a block mesh is laid out on its
// full voxel grid (voxels of removed box cells are holes: no equation, value
// zero), so every level addresses its neighbours by index arithmetic.  Level
// l + 1 aggregates 2x2x2 voxels of level l (ceil(n/2) aggregates per axis);
// its operator is the Galerkin product P^T A P with piecewise-constant P:
// face couplings summed across aggregate faces, diagonals and internal
// couplings summed into the diagonal.  One preconditioner application is a
// V-cycle: weighted-Jacobi sweeps before and after the scaled coarse
// correction, a dense inverse on the coarsest level.
//
// The solve: the FP64 residual r = b - M x of the cell field decides
// convergence (||r||2 <= tol ||b||2, the true residual, not a recurrence);
// each outer step scales r by a power of two into FP32, solves M d = r on the
// voxel grid with a flexible FP32 PCG (Polak-Ribiere beta) to a relative
// residual eta, and adds d to x in FP64.  FP64 work is one residual and one
// update per outer step; everything per inner iteration is FP32.
//
// The whole solve is one CUDA graph: an outer while-node around the inner
// while-node; the kernels that close each loop set its condition, with caps
// on the inner, total and outer iteration counts so that both loops end.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "hexmesh.hpp"

namespace pgd {

// Device scalars of one solve.
struct MgScalars {
    // outer (FP64 refinement)
    double rr, bb, lim, rr0, scale, inv_scale, eta;
    int done, converged, outer, total, maxit, pad0;
    // inner (FP32 PCG, scalars kept in FP64)
    double irr, ilim, rz, beta, alpha, qz;
    int idone, k;
    unsigned int ticket;
    unsigned int pad1;
};

// One level on the device.
struct MgLevel {
    int n[3];             // voxel grid
    int cyc[3];           // periodic axes
    int fac[3];           // aggregation factor towards the next level (1 or 2)
    long V;
    int uniform;          // every coupling between active voxels in direction f equals coef[f]
    float coef[6];
    float* diag = nullptr;      // V (1 on holes)
    float* inv = nullptr;       // V (0 on holes)
    float* off = nullptr;       // 6 x V (direction f = 2 axis + 1 for +), null when uniform
    float* b = nullptr;         // V: right-hand side at this level (level 0: the inner residual)
    float* x = nullptr;         // V
    float* t = nullptr;         // V: Jacobi ping-pong
};

struct MgSettings {
    int pre = 2, post = 2, coarsest = 512;
    double omega = 0.8, scale = 1.6;
};

class MultigridPCG {
   public:
    ~MultigridPCG();
    // Builds the hierarchy from the mesh and the FP64 operator (M = -lap);
    // returns false with a message if the mesh is not a block mesh whose
    // neighbours follow its grid.
    bool init(const pg::HexMesh& m, const std::vector<double>& Mdiag, const std::vector<double>& Moff,
              const MgSettings& set, std::string* msg);
    // Solves M x = b (device vectors over the cells) from the given x to
    // ||b - M x||2 <= tol ||b||2 within maxit inner iterations.  Results:
    // inner iterations, outer steps, initial and final r.r, b.b, converged.
    cudaError_t solve(const DMesh& dm, const double* b, double* x, double tol, int maxit, cudaStream_t s,
                      int* iters, int* outer, double* rr0, double* rr, double* bb, bool* converged);
    int levels() const { return int(lv_.size()); }
    int coarsest_cells() const { return nc_; }
    const MgLevel& level(int l) const { return lv_[l]; }
    int64_t launches = 0;          // kernels run by solve() (counted from the iteration counts)
    size_t device_bytes = 0;

   private:
    std::vector<MgLevel> lv_;
    MgSettings set_;
    int nc_ = 0;                   // active voxels of the coarsest level
    int* cidx_ = nullptr;          // their voxel ids
    float* cinv_ = nullptr;        // dense inverse, nc_ x nc_
    int* vox_ = nullptr;           // voxel of each cell
    int n_cells_ = 0;
    double* r64_ = nullptr;        // FP64 residual over the cells
    float *d_ = nullptr, *p_ = nullptr, *q_ = nullptr;  // inner vectors on the level-0 grid
    double* part_ = nullptr;
    long part_cap_ = 0;
    MgScalars* sc_ = nullptr;
    unsigned int* guard_ = nullptr;   // inner iterations of the solve, kept apart from the scalars
    MgScalars* sc_host_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    const double* graph_b_ = nullptr;
    double* graph_x_ = nullptr;
    double graph_tol_ = -1;
    int graph_maxit_ = -1;
    int inner_launches_ = 0, outer_launches_ = 0;
    std::vector<void*> dev_;

    template <class T>
    T* dalloc(size_t n);
    bool use_graph_ = true;         // PICGPU_MG_GRAPH=0: host-driven loops (kernel profilers)

    int vcycle(int l, cudaStream_t s);    // returns kernels launched; level 0 ends with r.z
    float* result(int l) const;
    int inner_iteration(cudaStream_t s, int maxit, cudaGraphConditionalHandle h_inner, int graph);
    void residual(const DMesh& dm, const double* b, double* x, int first, double tol, int maxit, cudaStream_t s,
                  cudaGraphConditionalHandle h_outer, int graph);
    cudaError_t build_graph(const DMesh& dm, const double* b, double* x, double tol, int maxit, cudaStream_t s);
    cudaError_t solve_eager(const DMesh& dm, const double* b, double* x, double tol, int maxit, cudaStream_t s);
};

}  // namespace pgd
