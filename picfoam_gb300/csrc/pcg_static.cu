// pcg_static.cu -- allocation-free variant of the Poisson PCG.
//
// picgpu_solve_ldu_noalloc runs the same PCG kernels as picgpu_solve_poisson
// (Jacobi preconditioner, fixed-order reductions) on a matrix and vectors the
// caller already holds in device memory.  Its working vectors live in one
// file-scope __device__ array instead of cudaMalloc'd buffers, so the call
// allocates nothing: it is meant for callers that cannot call cudaMalloc,
// e.g. a solver plugin hosted by a framework whose memory pool owns all
// device memory, or a time-critical loop where cudaMalloc's implicit
// device-wide synchronisation is not acceptable.
//
// The scratch array (kNoallocScratchDoubles doubles, about 3.2 MB) is
// created when the library is loaded on a device and stays there until the
// process exits; it bounds the problem to PICGPU_NOALLOC_MAX_CELLS cells.
// Every call on a device uses the same array and leaves the last call's
// contents in it, so calls whose GPU work overlaps (different host threads or
// different streams) race; serialise them.
#include <cstring>
#include <mutex>

#include "fields.h"
#include "picgpu.h"

namespace {

constexpr long kMaxCells = PICGPU_NOALLOC_MAX_CELLS;
constexpr long kMaxBlocks = (kMaxCells + pgd::kChunk - 1) / pgd::kChunk;
constexpr long kPartDoubles = 4 * kMaxBlocks + 8;
constexpr long kStateDoubles = 32;  // holds one pgd::PcgState (rounded up)
constexpr long kNoallocScratchDoubles = 6 * kMaxCells + kPartDoubles + kStateDoubles;
static_assert(sizeof(pgd::PcgState) <= kStateDoubles * sizeof(double), "state does not fit");

// The scratch: dinv | r | u | p | s | w | partial sums | PCG state.
static __device__ __align__(256) double g_pcg_scratch[kNoallocScratchDoubles];

// Device address of g_pcg_scratch per device, filled on the first call made
// with that device current (cudaGetSymbolAddress must not run inside a stream
// capture, so make the first call on each device before capturing).
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

__global__ void reciprocal_kernel(const double* __restrict__ a, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = 1.0 / a[i];
}

}  // namespace

extern "C" picgpu_status picgpu_solve_ldu_noalloc(int n_cells, const double* diag, const double* off,
                                                  const int32_t* nbr, const double* b, double* x,
                                                  double tol, int max_iter, int* iterations,
                                                  double* residual, void* stream) {
    if (n_cells <= 0 || !diag || !off || !nbr || !b || !x || !(tol > 0) || max_iter <= 0)
        return PICGPU_INVALID_ARG;
    if (n_cells > kMaxCells) return PICGPU_CAPACITY;  // scratch holds PICGPU_NOALLOC_MAX_CELLS cells
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PICGPU_CUDA_ERROR;
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_pcg_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return PICGPU_CUDA_ERROR;
            }
            g_scratch_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long n = n_cells;
    double* dinv = scratch;
    double* r = dinv + n;
    double* u = r + n;
    double* p = u + n;
    double* sv = u + 2 * n;
    double* w = u + 3 * n;
    double* part = scratch + 6 * kMaxCells;
    auto* st = reinterpret_cast<pgd::PcgState*>(part + kPartDoubles);
    // the state carries the reduction ticket, which must start at zero
    if (cudaMemsetAsync(st, 0, sizeof(pgd::PcgState), s) != cudaSuccess) return PICGPU_CUDA_ERROR;
    reciprocal_kernel<<<int((n + 255) / 256), 256, 0, s>>>(diag, dinv, n_cells);
    pgd::DMesh m{};
    m.n_cells = n_cells;
    m.Mdiag = diag;
    m.Moff = off;
    m.nbr = nbr;
    m.dinv = dinv;
    pgd::launch_pcg_init(m, b, x, r, u, w, part, st, tol, s);
    pgd::PcgState h{};
    // a launch error of the set-up kernels must not pass for convergence when
    // the start guess already meets the tolerance and no iteration runs
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    int k = 1, batch = 4;
    while (!h.done && k <= max_iter) {
        for (int j = 0; j < batch && k <= max_iter; ++j, ++k)
            pgd::launch_pcg_iteration(m, x, r, u, w, p, sv, part, st, max_iter, s);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return PICGPU_CUDA_ERROR;
        batch = batch < 32 ? 2 * batch : 32;
    }
    if (iterations) *iterations = h.iters;
    if (residual) *residual = h.bb > 0 ? std::sqrt(h.rr / h.bb) : 0.0;
    return h.converged ? PICGPU_OK : PICGPU_PCG_NOT_CONVERGED;
}
