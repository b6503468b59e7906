// mg.h -- flexible FP64 PCG with an FP32 aggregation-multigrid preconditioner.
//
// The Poisson operator M (SPD, -laplacian) of a block mesh is laid out on its
// full voxel grid (voxels of removed box cells are holes: no equation, value
// zero), so every level addresses its neighbours by index arithmetic.  Level
// l + 1 aggregates 2x2x2 voxels of level l (ceil(n/2) aggregates per axis);
// its operator is the Galerkin product P^T A P with piecewise-constant P:
// face couplings summed across aggregate faces, diagonals and internal
// couplings summed into the diagonal.  One preconditioner application is a
// V-cycle in FP32: weighted-Jacobi sweeps before and after the (scaled) coarse
// correction, a dense inverse on the coarsest level.  The outer iteration is
// an FP64 flexible PCG (Polak-Ribiere beta, so the FP32 rounding of the
// V-cycle cannot stall it) with fixed-order reductions, and it stops on
// ||b - M x||2 <= tol ||b||2 exactly as the Jacobi PCG does.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "hexmesh.hpp"

namespace pgd {

// Device scalars of one solve.
struct MgScalars {
    double rz, beta, alpha, rr, bb, lim, rr0, pad0;
    int done, converged, k, maxit;
    unsigned int ticket;
    unsigned int pad1[3];
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
    float* b = nullptr;         // V: right-hand side at this level
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
    // ||r||2 <= tol ||b||2 within maxit iterations.  Results: iterations,
    // initial and final r.r, b.b, converged.
    cudaError_t solve(const DMesh& dm, const double* b, double* x, double tol, int maxit, cudaStream_t s,
                      int* iters, double* rr0, double* rr, double* bb, bool* converged);
    int levels() const { return int(lv_.size()); }
    int coarsest_cells() const { return nc_; }
    const MgLevel& level(int l) const { return lv_[l]; }
    int64_t launches = 0;          // kernels launched by solve()
    size_t device_bytes = 0;

   private:
    std::vector<MgLevel> lv_;
    MgSettings set_;
    int nc_ = 0;                   // active voxels of the coarsest level
    int* cidx_ = nullptr;          // their voxel ids
    float* cinv_ = nullptr;        // dense inverse, nc_ x nc_
    int* vox_ = nullptr;           // voxel of each cell
    int n_cells_ = 0;
    double *r_ = nullptr, *z_ = nullptr, *p_ = nullptr, *q_ = nullptr, *part_ = nullptr;
    MgScalars* sc_ = nullptr;
    MgScalars* sc_host_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    const double* graph_b_ = nullptr;
    double* graph_x_ = nullptr;
    int graph_launches_ = 0;
    std::vector<void*> dev_;

    template <class T>
    T* dalloc(size_t n);
    int vcycle(int l, cudaStream_t s);                       // returns kernels launched
    float* result(int l) const;
    int iteration(const DMesh& dm, double* x, cudaStream_t s);
};

}  // namespace pgd
