// learned.cu -- the learned warm start of the Poisson PCG.
//
// picFoam's ElectroStaticSolver starts each solve from the previous
// potential (ElectroStaticSolver.C:61-64).  Here, after a training phase,
// the start is phi_prev + alpha d with d the U-Net's prediction of the
// potential increment from the start residual r = b - M phi_prev (the
// right-hand-side increment: charge change and floating-patch updates), and
// alpha = (d . r) / (d . M d) the A-norm-optimal step along d, so the start
// is never worse than phi_prev in the energy norm.  The FP64 PCG then runs to
// the unchanged tolerance: the net only moves the starting point.
//
// Training data are the pairs the plain solver emits during the first
// train_steps solves: input r / rms(r) and the domain mask on the cell grid,
// target (phi_new - phi_prev) / rms(r) * c0 with c0 fixed from the first
// pair, so targets are O(1).  The net is bias-free and ReLU, hence
// positively homogeneous, and the scaling is undone exactly at inference.
#include <cmath>

#include "learned.h"

namespace pgd {
namespace {

constexpr int kDotBlocks = 304;

__device__ __forceinline__ double apply_row(const DMesh& m, const double* __restrict__ x, int c) {
    double s = m.Mdiag[c] * x[c];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const int nb = m.nbr[6 * size_t(c) + f];
        if (nb >= 0) s = fma(m.Moff[6 * size_t(c) + f], x[nb], s);
    }
    return s;
}

__global__ void residual_kernel(DMesh m, const double* __restrict__ b, const double* __restrict__ x,
                                double* __restrict__ r) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < m.n_cells) r[c] = b[c] - apply_row(m, x, c);
}

__global__ void apply_kernel(DMesh m, const double* __restrict__ x, double* __restrict__ y) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < m.n_cells) y[c] = apply_row(m, x, c);
}

// Deterministic dot product: a fixed grid of kDotBlocks blocks (grid-stride
// partial sums, fixed block tree), then one block sums the partials in order.
__global__ void dot_partial_kernel(const double* __restrict__ a, const double* __restrict__ b, long n,
                                   double* __restrict__ part) {
    __shared__ double s[256];
    double v = 0.0;
    for (long i = long(blockIdx.x) * 256 + threadIdx.x; i < n; i += long(gridDim.x) * 256) v = fma(a[i], b[i], v);
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void dot_final_kernel(const double* __restrict__ part, int n, double* out) {
    __shared__ double s[256];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) v += part[i];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

// Input and output scales from r . r (and c0).
__global__ void scales_kernel(WsScalars* sc, int n) {
    const double rms = sqrt(sc->rr / double(n));
    sc->inv_rms = rms > 0 ? 1.0 / rms : 0.0;
    sc->scale = sc->c0 > 0 ? rms / sc->c0 : 0.0;
}

__global__ void to_grid_kernel(int n, const int* __restrict__ vox, const double* __restrict__ r, const WsScalars* sc,
                               float* __restrict__ in) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) in[2 * size_t(vox[c])] = float(r[c] * sc->inv_rms);
}

__global__ void from_grid_kernel(int n, const int* __restrict__ vox, const float* __restrict__ out,
                                 const WsScalars* sc, double* __restrict__ d) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) d[c] = double(out[vox[c]]) * sc->scale;
}

__global__ void alpha_kernel(WsScalars* sc) {
    const double a = sc->dr / sc->dmd;
    sc->alpha = (sc->dmd > 0 && isfinite(a)) ? a : 0.0;
}

__global__ void axpy_kernel(int n, const WsScalars* sc, const double* __restrict__ d, double* __restrict__ x) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) x[c] = fma(sc->alpha, d[c], x[c]);
}

__global__ void diff_kernel(int n, const double* __restrict__ x, const double* __restrict__ prev,
                            double* __restrict__ e) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) e[c] = x[c] - prev[c];
}

// One training pair in grid layout: input channel 0 and the target.
__global__ void sample_kernel(int n, const int* __restrict__ vox, const double* __restrict__ r,
                              const double* __restrict__ e, const WsScalars* sc, float* __restrict__ in,
                              float* __restrict__ tgt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int v = vox[c];
    in[2 * size_t(v)] = float(r[c] * sc->inv_rms);
    tgt[v] = float(e[c] * sc->inv_rms * sc->c0);
}

__global__ void mask_channel_kernel(long V, const float* __restrict__ mask, float* __restrict__ in) {
    const long v = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v < V) {
        in[2 * v] = 0.f;
        in[2 * v + 1] = mask[v];
    }
}

unsigned blocks(long n) { return unsigned((n + 255) / 256); }

}  // namespace

template <class T>
T* LearnedWarmStart::alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    allocs_.push_back(p);
    return static_cast<T*>(p);
}

LearnedWarmStart::~LearnedWarmStart() {
    for (void* p : allocs_) cudaFree(p);
    if (sc_host_) cudaFreeHost(sc_host_);
}

int LearnedWarmStart::init(const picgpu_learned& cfg, uint64_t seed, int n_cells, const int grid[3],
                           const std::vector<int>& ijk, cudaStream_t s, std::string* msg) {
    cfg_ = cfg;
    if (cfg_.train_steps <= 0) cfg_.train_steps = 500;
    if (cfg_.train_iters <= 0) cfg_.train_iters = 4;
    if (cfg_.replay <= 0) cfg_.replay = 16;
    if (!(cfg_.lr > 0)) cfg_.lr = 1e-3;
    if (cfg_.refine < 0 || cfg_.refine > 3) {
        *msg = "learned warm start: refine must be 0..3";
        return PICGPU_INVALID_ARG;
    }
    if (!UNet::grid_supported(grid[0], grid[1], grid[2])) {
        *msg = "learned warm start: the block mesh needs cell counts that are multiples of 4 with "
               "n0*n1*n2/64 a multiple of 128";
        return PICGPU_NOT_SUPPORTED;
    }
    const int e = net_.init(grid[0], grid[1], grid[2], seed, msg);
    if (e) return e == 2 ? PICGPU_OOM : PICGPU_CUDA_ERROR;
    n_cells_ = n_cells;
    V_ = net_.voxels();
    rng_ = seed ^ 0xD1B54A32D192ED03ull;
    std::vector<int> vox(n_cells);
    std::vector<float> mask(V_, 0.f);
    for (int c = 0; c < n_cells; ++c) {
        vox[c] = ijk[3 * size_t(c)] + grid[0] * (ijk[3 * size_t(c) + 1] + grid[1] * ijk[3 * size_t(c) + 2]);
        mask[vox[c]] = 1.f;
    }
    vox_ = alloc<int>(n_cells);
    mask_ = alloc<float>(V_);
    rep_in_ = alloc<float>(size_t(cfg_.replay) * V_ * 2);
    rep_tgt_ = alloc<float>(size_t(cfg_.replay) * V_);
    r_ = alloc<double>(n_cells);
    d_ = alloc<double>(n_cells);
    md_ = alloc<double>(n_cells);
    prev_ = alloc<double>(n_cells);
    part_ = alloc<double>(kDotBlocks);
    sc_ = alloc<WsScalars>(1);
    if (!vox_ || !mask_ || !rep_in_ || !rep_tgt_ || !r_ || !d_ || !md_ || !prev_ || !part_ || !sc_ ||
        cudaMallocHost(&sc_host_, sizeof(WsScalars)) != cudaSuccess) {
        *msg = "learned warm start: device allocation failed";
        return PICGPU_OOM;
    }
    if (cudaMemcpy(vox_, vox.data(), vox.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(mask_, mask.data(), mask.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(sc_, 0, sizeof(WsScalars)) != cudaSuccess) {
        *msg = "learned warm start: upload failed";
        return PICGPU_CUDA_ERROR;
    }
    // the mask channel of every replay input and of the net's input
    for (int k = 0; k < cfg_.replay; ++k)
        mask_channel_kernel<<<blocks(V_), 256, 0, s>>>(V_, mask_, rep_in_ + size_t(k) * V_ * 2);
    mask_channel_kernel<<<blocks(V_), 256, 0, s>>>(V_, mask_, net_.input());
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "learned warm start: initialisation failed";
        return PICGPU_CUDA_ERROR;
    }
    return PICGPU_OK;
}

void LearnedWarmStart::dot(const double* a, const double* b, double* out, cudaStream_t s) {
    dot_partial_kernel<<<kDotBlocks, 256, 0, s>>>(a, b, n_cells_, part_);
    dot_final_kernel<<<1, 256, 0, s>>>(part_, kDotBlocks, out);
    launches += 2;
}

void LearnedWarmStart::residual(const DMesh& m, const double* b, const double* x, cudaStream_t s) {
    residual_kernel<<<blocks(n_cells_), 256, 0, s>>>(m, b, x, r_);
    dot(r_, r_, &sc_->rr, s);
    launches += 1;
}

cudaError_t LearnedWarmStart::net_pass(const DMesh& m, const double* b, double* phi, cudaStream_t s) {
    (void)b;
    scales_kernel<<<1, 1, 0, s>>>(sc_, n_cells_);
    to_grid_kernel<<<blocks(n_cells_), 256, 0, s>>>(n_cells_, vox_, r_, sc_, net_.input());
    cudaError_t e = net_.forward(s);
    if (e != cudaSuccess) return e;
    from_grid_kernel<<<blocks(n_cells_), 256, 0, s>>>(n_cells_, vox_, net_.output(), sc_, d_);
    apply_kernel<<<blocks(n_cells_), 256, 0, s>>>(m, d_, md_);
    dot(d_, r_, &sc_->dr, s);
    dot(d_, md_, &sc_->dmd, s);
    alpha_kernel<<<1, 1, 0, s>>>(sc_);
    axpy_kernel<<<blocks(n_cells_), 256, 0, s>>>(n_cells_, sc_, d_, phi);
    launches += 6;
    return cudaGetLastError();
}

cudaError_t LearnedWarmStart::before(const DMesh& m, const double* b, double* phi, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(prev_, phi, size_t(n_cells_) * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    residual(m, b, phi, s);
    dot(b, b, &sc_->bb, s);
    cudaMemcpyAsync(&sc_->plain_rr, &sc_->rr, sizeof(double), cudaMemcpyDeviceToDevice, s);
    active = 0;
    if (!trained() || !have_c0_ || fallback) return cudaGetLastError();
    for (int pass = 0; pass <= cfg_.refine; ++pass) {
        if (pass > 0) residual(m, b, phi, s);
        if ((e = net_pass(m, b, phi, s)) != cudaSuccess) return e;
    }
    active = 1;
    return cudaGetLastError();
}

cudaError_t LearnedWarmStart::after(const DMesh& m, const double* phi, int iterations, cudaStream_t s) {
    (void)m;
    cudaError_t e;
    if (active) {
        // does the net cut iterations?  Window of 20 solves against the
        // plain solves of the training phase; off for good if not.
        net_iters_ += iterations;
        if (++net_n_ == 20) {
            if (plain_n_ > 0 && net_iters_ / net_n_ > 0.98 * (plain_iters_ / plain_n_)) fallback = 1;
            net_iters_ = 0.0;
            net_n_ = 0;
        }
    }
    if (!trained()) {
        // the pair (r(phi_prev), phi - phi_prev); r_ still holds r(phi_prev)
        // because a solve in the training phase has no net pass
        diff_kernel<<<blocks(n_cells_), 256, 0, s>>>(n_cells_, phi, prev_, d_);
        dot(d_, d_, &sc_->ee, s);
        launches += 1;
        if ((e = cudaMemcpyAsync(sc_host_, sc_, sizeof(WsScalars), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return e;
        const WsScalars h = *sc_host_;
        // a solve that starts far from its solution (the first one, from
        // zero) is not a warm-start pair
        const bool warm = h.bb > 0 && h.rr > 0 && h.ee > 0 && h.plain_rr <= 0.25 * h.bb;
        if (warm) {
            if (!have_c0_) {
                const double c0 = std::sqrt(h.rr / h.ee);
                if ((e = cudaMemcpyAsync(&sc_->c0, &c0, sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                    (e = cudaStreamSynchronize(s)) != cudaSuccess)
                    return e;
                have_c0_ = true;
            }
            scales_kernel<<<1, 1, 0, s>>>(sc_, n_cells_);
            sample_kernel<<<blocks(n_cells_), 256, 0, s>>>(n_cells_, vox_, r_, d_, sc_,
                                                           rep_in_ + size_t(head_) * V_ * 2,
                                                           rep_tgt_ + size_t(head_) * V_);
            head_ = (head_ + 1) % cfg_.replay;
            samples = std::min(samples + 1, cfg_.replay);
            launches += 2;
            for (int it = 0; it < cfg_.train_iters; ++it) {
                rng_ += 0x9E3779B97F4A7C15ull;
                uint64_t z = rng_;
                z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
                z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
                const int k = int((z ^ (z >> 31)) % uint64_t(samples));
                // ring slot k counted back from the newest
                const int slot = ((head_ - 1 - k) % cfg_.replay + cfg_.replay) % cfg_.replay;
                if ((e = cudaMemcpyAsync(net_.input(), rep_in_ + size_t(slot) * V_ * 2, size_t(V_) * 2 * sizeof(float),
                                         cudaMemcpyDeviceToDevice, s)) != cudaSuccess ||
                    (e = net_.forward(s)) != cudaSuccess ||
                    (e = net_.loss_and_grad(rep_tgt_ + size_t(slot) * V_, mask_, s)) != cudaSuccess ||
                    (e = net_.backward(s)) != cudaSuccess || (e = net_.adam(float(cfg_.lr), s)) != cudaSuccess)
                    return e;
            }
            if ((e = net_.read_loss(&loss, s)) != cudaSuccess) return e;
            plain_iters_ += iterations;
            ++plain_n_;
            ++solves_;
        }
    }
    if ((e = cudaMemcpyAsync(sc_host_, sc_, sizeof(WsScalars), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return e;
    alpha = active ? sc_host_->alpha : 0.0;
    plain_residual = sc_host_->bb > 0 ? std::sqrt(sc_host_->plain_rr / sc_host_->bb) : 0.0;
    bool timed_out = false;
    if ((e = net_.check_error(&timed_out, s)) != cudaSuccess) return e;
    return timed_out ? cudaErrorLaunchTimeout : cudaSuccess;
}

}  // namespace pgd
