// learned.h -- the learned warm start of the Poisson PCG inside picgpu_step.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "unet_net.h"

namespace pgd {

// Scalars the warm-start kernels share on the device.
struct WsScalars {
    double rr;       // r . r of the residual being processed
    double bb;       // b . b
    double dr;       // d . r
    double dmd;      // d . M d
    double alpha;    // line-search factor of the last pass
    double inv_rms;  // sqrt(n / r.r): input scale of the net
    double scale;    // rms(r) / c0: output scale of the net
    double c0;       // rms(r) / rms(e) of the first training pair
    double ee;       // e . e
    double plain_rr; // r . r of the previous potential (the plain guess)
};

class LearnedWarmStart {
   public:
    // grid: the block mesh's cell counts; ijk: 3 per cell.  0 on success.
    int init(const picgpu_learned& cfg, uint64_t seed, int n_cells, const int grid[3], const std::vector<int>& ijk,
             cudaStream_t s, std::string* msg);
    // Before the PCG: residual of phi, a copy of phi, and (once trained) the
    // net's increment(s) added to phi with the A-norm line search.
    cudaError_t before(const DMesh& m, const double* b, double* phi, cudaStream_t s);
    // After the PCG: during training, store (residual, increment) and train.
    // iterations: the PCG iterations the solve just took.
    cudaError_t after(const DMesh& m, const double* phi, int iterations, cudaStream_t s);
    bool trained() const { return solves_ >= cfg_.train_steps; }

    double loss = 0.0, alpha = 0.0, plain_residual = 0.0;
    int active = 0;
    int samples = 0;
    int fallback = 0;  // 1 once the net was switched off for not cutting iterations
    int64_t launches = 0;

   private:
    picgpu_learned cfg_{};
    UNet net_;
    int n_cells_ = 0;
    long V_ = 0;
    int* vox_ = nullptr;          // voxel of each cell
    float* mask_ = nullptr;       // [V]: 1 on cells
    float* rep_in_ = nullptr;     // replay inputs [R][V][2]
    float* rep_tgt_ = nullptr;    // replay targets [R][V]
    double *r_ = nullptr, *d_ = nullptr, *md_ = nullptr, *prev_ = nullptr, *part_ = nullptr;
    WsScalars* sc_ = nullptr;
    WsScalars* sc_host_ = nullptr;
    std::vector<void*> allocs_;
    int solves_ = 0;
    int head_ = 0;
    double plain_iters_ = 0.0;   // PCG iterations of the warm training solves (previous-potential start)
    int plain_n_ = 0;
    double net_iters_ = 0.0;     // of the current window of net-started solves
    int net_n_ = 0;
    uint64_t rng_ = 0;
    bool have_c0_ = false;

    template <class T>
    T* alloc(size_t n);
    void dot(const double* a, const double* b, double* out, cudaStream_t s);
    void residual(const DMesh& m, const double* b, const double* x, cudaStream_t s);
    cudaError_t net_pass(const DMesh& m, const double* b, double* phi, cudaStream_t s);

   public:
    ~LearnedWarmStart();
};

}  // namespace pgd
