// library.cu -- the picgpu C ABI: context, device memory, step orchestration.
//
// A context holds one PIC/MCC case resident on the current CUDA device.
// picgpu_step runs the PICCloud::evolve sequence
// (PICMCCFVM/clouds/Templates/PICCloud/PICCloud.C:1426-1471) as a chain of
// kernels on the context's stream:
//
//   zero charge accumulators
//   move (push + track + patch + deposit), one launch per species
//   collisions (Coulomb, electron-neutral MCC) on the cell-sorted store
//   charge update -> rho            (calculateFields, PICCloud.C:587-695)
//   floating patches: sigma, g      (preUpdate_Boundary)
//   Poisson PCG, E, point E         (ElectroStaticSolver::solveFields)
//
// Nothing returns to the host inside a step except the PCG convergence flag
// and the per-step counters.
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "collide.h"
#include "fields.h"
#include "emission.hpp"
#include "freestream.hpp"
#include "init.h"
#include "hexmesh.hpp"
#include "kernels.h"
#include "learned.h"
#include "mg.h"
#include "particles.h"
#include "picgpu.h"
#include "picgpu_ensemble.h"
#include "picgpu_init.h"

using pgd::DMesh;

struct picgpu_mesh {
    pg::HexMesh m;
};

namespace {

constexpr double kMu0 = 4.0 * 3.14159265358979323846 * 1e-7;
constexpr int kGraphIters = 8;  // PCG iterations per graph replay
constexpr double kCl = 299792458.0;

struct SpeciesBuf {
    long n = 0;      // used slots (removed particles keep tet = -1 until compaction)
    long alive = 0;  // particles in the used slots that are not removed
    long cap = 0;
    int cur = 0;     // active buffer of the double-buffered store
    int32_t* tet[2] = {nullptr, nullptr};
    double* y64[2][3] = {};
    double* u64[2][3] = {};
    float* y32[2][3] = {};
    float* u32[2][3] = {};
    // per-parcel nParticle and chargeModifier (both halves), allocated when
    // a caller sets them or a model (PairMerging, Perez ionisation) needs them
    bool attrs = false;
    double* nw[2] = {nullptr, nullptr};
    int32_t* zq[2] = {nullptr, nullptr};
};

// Host <-> device copies of caller (pageable) arrays through a pinned ring of
// two slots: host threads copy chunk k into a slot while the DMA engine moves
// chunk k - 1, so the copy runs at the host's memcpy bandwidth over all its
// cores instead of through the driver's single bounce buffer.
// Host-side copy workers of the staging ring: started once with the
// context, they wait on a condition variable; a copy splits into one segment
// per worker plus one for the calling thread.
class CopyPool {
  public:
    void start(unsigned workers) {
        for (unsigned k = 0; k < workers; ++k) th_.emplace_back([this, k] { run(k + 1); });
    }
    void stop() {
        {
            std::lock_guard<std::mutex> g(m_);
            quit_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
        th_.clear();
        quit_ = false;
    }
    void copy(char* dst, const char* src, size_t n) {
        const unsigned parts = unsigned(th_.size()) + 1;
        if (th_.empty() || n < (size_t(4) << 20)) {
            std::memcpy(dst, src, n);
            return;
        }
        {
            std::lock_guard<std::mutex> g(m_);
            dst_ = dst;
            src_ = src;
            n_ = n;
            part_ = (n + parts - 1) / parts;
            pending_ = unsigned(th_.size());
            ++gen_;
        }
        cv_.notify_all();
        segment(0);
        std::unique_lock<std::mutex> g(m_);
        done_.wait(g, [this] { return pending_ == 0; });
    }

  private:
    void segment(unsigned k) {
        const size_t a = k * part_, b = std::min(n_, a + part_);
        if (a < b) std::memcpy(dst_ + a, src_ + a, b - a);
    }
    void run(unsigned k) {
        unsigned seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return quit_ || gen_ != seen; });
                if (quit_) return;
                seen = gen_;
            }
            segment(k);
            {
                std::lock_guard<std::mutex> g(m_);
                if (--pending_ == 0) done_.notify_all();
            }
        }
    }
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    char* dst_ = nullptr;
    const char* src_ = nullptr;
    size_t n_ = 0, part_ = 0;
    unsigned gen_ = 0, pending_ = 0;
    bool quit_ = false;
};

struct HostStager {
    static constexpr size_t kSlot = size_t(64) << 20;
    char* pinned = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool ready = false;
    CopyPool pool;

    bool init() {
        if (ready) return true;
        if (cudaMallocHost(&pinned, 2 * kSlot) != cudaSuccess) return false;
        for (int k = 0; k < 2; ++k)
            if (cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming) != cudaSuccess) return false;
        const unsigned t = std::max(1u, std::min(std::thread::hardware_concurrency(), 16u));
        pool.start(t - 1);
        ready = true;
        return true;
    }
    void release() {
        if (ready) pool.stop();
        if (pinned) cudaFreeHost(pinned);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        pinned = nullptr;
        ev[0] = ev[1] = nullptr;
        ready = false;
    }
    void par_copy(char* dst, const char* src, size_t n) { pool.copy(dst, src, n); }
    // page-locked caller memory (picgpu_host_alloc, cudaHostRegister ...)
    static bool pinned_host(const void* p) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return a.type == cudaMemoryTypeHost;
    }
    cudaError_t upload(void* dev, const void* host, size_t n, cudaStream_t s) {
        if (n < (size_t(8) << 20) || pinned_host(host) || !init())
            return cudaMemcpyAsync(dev, host, n, cudaMemcpyHostToDevice, s);
        const char* src = static_cast<const char*>(host);
        char* dst = static_cast<char*>(dev);
        int k = 0;
        for (size_t off = 0; off < n; off += kSlot, k ^= 1) {
            const size_t len = std::min(kSlot, n - off);
            cudaError_t e = cudaEventSynchronize(ev[k]);  // the slot's previous DMA is done
            if (e != cudaSuccess) return e;
            par_copy(pinned + k * kSlot, src + off, len);
            if ((e = cudaMemcpyAsync(dst + off, pinned + k * kSlot, len, cudaMemcpyHostToDevice, s))) return e;
            if ((e = cudaEventRecord(ev[k], s))) return e;
        }
        return cudaSuccess;
    }
    cudaError_t download(void* host, const void* dev, size_t n, cudaStream_t s) {
        if (n < (size_t(8) << 20) || pinned_host(host) || !init()) {
            cudaError_t e = cudaMemcpyAsync(host, dev, n, cudaMemcpyDeviceToHost, s);
            return e ? e : cudaStreamSynchronize(s);
        }
        char* dst = static_cast<char*>(host);
        const char* src = static_cast<const char*>(dev);
        const size_t nch = (n + kSlot - 1) / kSlot;
        cudaError_t e;
        // DMA of chunk k + 1 runs while the host drains chunk k
        if ((e = cudaMemcpyAsync(pinned, src, std::min(kSlot, n), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaEventRecord(ev[0], s))) return e;
        for (size_t k = 0; k < nch; ++k) {
            const int slot = int(k & 1);
            if (k + 1 < nch) {
                const size_t off = (k + 1) * kSlot, len = std::min(kSlot, n - off);
                if ((e = cudaMemcpyAsync(pinned + (slot ^ 1) * kSlot, src + off, len, cudaMemcpyDeviceToHost, s)))
                    return e;
                if ((e = cudaEventRecord(ev[slot ^ 1], s))) return e;
            }
            if ((e = cudaEventSynchronize(ev[slot]))) return e;
            const size_t off = k * kSlot, len = std::min(kSlot, n - off);
            par_copy(dst + off, pinned + slot * kSlot, len);
        }
        return cudaSuccess;
    }
};

// A SimpleInjection boundary model on one patch.
struct Injector {
    picgpu_injection cfg{};
    double remainder[PICGPU_MAX_SPECIES] = {};   // particleRemainder_
    int n_tri = 0;
    double area = 0.0;
    double* tri_cum = nullptr;
    int* tri_cell = nullptr;
    int* tri_tet = nullptr;
    double* tri_normal = nullptr;
    double* tri_fc = nullptr;
    // EmissionModel (picgpu_set_emission) on the patch
    picgpu_emission em{};
    double em_j = 0.0;             // thermionic current density [A/m^2]
    double em_remainder = 0.0;     // pRemainder_
    int* em_faces = nullptr;       // Fowler-Nordheim: the patch's boundary faces
    int em_n_faces = 0;
};

// FreeStream boundary model: per-face tables and accumulators on the device.
struct FsInjector {
    picgpu_freestream cfg{};
    pg::FreeStreamFaces F;          // host copy of the face tables
    int* cell = nullptr;
    int* tet0 = nullptr;
    double *frac0 = nullptr, *n_in = nullptr, *t1 = nullptr, *t2 = nullptr, *add = nullptr, *s = nullptr;
    double* acc = nullptr;          // n_faces * n_species
    int* counts = nullptr;          // n_faces
    long long* offsets = nullptr;   // n_faces + 1
    long long* sums = nullptr;      // scan scratch
};

struct EventPair {
    cudaEvent_t a, b;
    int phase;
};

}  // namespace

struct picgpu_ctx {
    std::string err;
    picgpu_config cfg{};
    pg::HexMesh m;
    cudaStream_t stream = nullptr;
    int device = 0, sm_count = 148;
    std::vector<void*> allocs;
    DMesh dm{};
    pgd::TetConst tc{};
    pgd::PatchConst pc{};
    SpeciesBuf sp[PICGPU_MAX_SPECIES];
    bool mixed = false;
    double *phi = nullptr, *rho = nullptr, *E = nullptr, *Ept = nullptr, *Eb = nullptr;
    float *E32 = nullptr, *Ept32 = nullptr;
    double *cc_data = nullptr, *vtx_data = nullptr;
    long long *cc_fix = nullptr, *vtx_fix = nullptr;
    unsigned long long* acc9 = nullptr;   // FP32 form: per-species fixed-point deposit, 9 slots per cell
    float4* Ec4 = nullptr;                // FP32 form: E per cell, centre + 8 corners
    pgd::Tables32* t32 = nullptr;         // FP32 form: this mesh's move tables (device)
    double* Bc = nullptr;                 // per-cell magnetic field (3 n_cells), null: uniform cfg.B
    float4* Bc4 = nullptr;                // its FP32 copy
    float cell_dth[3] = {0, 0, 0};        // FP32 in-cell mover: dt / cell size per axis (0: empty axis)
    float cell_keep[3] = {1, 1, 1};       // 0 on empty axes
    int* xq_count = nullptr;              // FP32 form: crossing-queue counts and starts per mover block
    int* xq_start = nullptr;
    int xq_cap = 0;
    double *qconv = nullptr, *sigma = nullptr, *grad_bc = nullptr;
    pgd::CircuitParams circ{};            // circuit model (model NONE: no circuit)
    pg::CircuitState* circ_state = nullptr;
    double *b = nullptr, *r = nullptr, *z = nullptr, *p[2] = {nullptr, nullptr}, *q = nullptr,
           *part = nullptr;
    pgd::PcgState* st = nullptr;
    pgd::PcgState* st_host = nullptr;
    pgd::MoveCounters* counters = nullptr;
    pgd::MoveCounters* counters_host = nullptr;
    double* diag = nullptr;
    double fix_scale = 1.0;
    bool rotation = false;
    long long step_index = 0;
    // compaction / sort scratch
    int* scan_buf = nullptr;
    long scan_cap = 0;
    pgd::CollideState coll{};
    // profiling
    bool profiling = false;
    std::vector<EventPair> pending;
    std::vector<cudaEvent_t> free_events;
    double phase_ms[PICGPU_PHASE_COUNT] = {};
    int64_t phase_launches[PICGPU_PHASE_COUNT] = {};
    int64_t launches = 0;
    picgpu_step_stats acc{};
    cudaEvent_t timer[2] = {nullptr, nullptr};
    cudaGraphExec_t pcg_graph = nullptr;
    double pcg_r0 = 0.0;  // ||b - A x0|| / ||b|| of the last solve's start guess
    std::unique_ptr<pgd::LearnedWarmStart> ws;  // learned warm start (cfg.learned.enabled)
    std::unique_ptr<pgd::MultigridPCG> mg;      // multigrid-preconditioned PCG (cfg.pcg_precond)
    int mg_outer = 0;                           // refinement steps of the last multigrid solve
    double* tet_vol = nullptr;                  // 12 tet volumes per geometry class (initial conditions)
    std::vector<Injector> injectors;            // SimpleInjection boundary models
    std::vector<FsInjector> freestreams;        // FreeStream boundary models
    std::vector<Injector> emitters;             // EmissionModels
    double* em_sum = nullptr;                   // Fowler-Nordheim patch current (device scalar)
    int* inj_err = nullptr;                     // an emitted parcel could not be located
    // row-major host arrays staged on the device (set/get_particles)
    int32_t* rows_tet = nullptr;
    double* rows_y = nullptr;
    double* rows_u = nullptr;
    size_t rows_cap = 0;
    int* inj_flag = nullptr;                    // device flag of the row checks
    HostStager stager;                          // pinned ring for caller arrays
    // batched ensembles and graph-stepped runs
    int n_cases = 1;
    int* n_dev = nullptr;          // species counts on the device (graph steps)
    int* first_dev = nullptr;      // counts before this step's secondaries
    unsigned* step_dev = nullptr;  // step index read by the collision kernels
    struct GraphEntry {
        uint64_t key;
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> graphs;
    uint64_t graph_sig = 0;        // signature of the buffers the cached graphs address
    cudaEvent_t replay_ev[2] = {nullptr, nullptr};  // the tuner's replay timing (not the user timer)
    int move_bps = 5;              // FP32 move kernel: blocks per SM
    bool tuned = false;
    std::vector<double> tune_ms;
    long long last_sort = -(1LL << 40);  // graph steps re-sort on their first replay
};

picgpu_status pgd_collisions(picgpu_ctx* c, picgpu_step_stats* stats);

namespace {

picgpu_status fail(picgpu_ctx* c, cudaError_t e, const char* what, int line) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "CUDA error %s (%s) at library.cu:%d: %s", cudaGetErrorName(e),
                  cudaGetErrorString(e), line, what);
    c->err = buf;
    return PICGPU_CUDA_ERROR;
}

#define CK(call)                                               \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return fail(c, e_, #call, __LINE__); \
    } while (0)

picgpu_status bad(picgpu_ctx* c, picgpu_status s, const std::string& msg) {
    c->err = msg;
    return s;
}

template <class T>
picgpu_status dalloc(picgpu_ctx* c, T** out, size_t count) {
    void* ptr = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c->err = "device allocation of " + std::to_string(bytes) + " bytes failed";
        return PICGPU_OOM;
    }
    c->allocs.push_back(ptr);
    *out = static_cast<T*>(ptr);
    return PICGPU_OK;
}

template <class T>
picgpu_status upload(picgpu_ctx* c, T** out, const std::vector<T>& v) {
    picgpu_status s = dalloc(c, out, v.size());
    if (s) return s;
    if (!v.empty()) CK(cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PICGPU_OK;
}

void dfree(picgpu_ctx* c, void* ptr) {
    if (!ptr) return;
    for (auto& a : c->allocs)
        if (a == ptr) { cudaFree(a); a = nullptr; }
}

// ------------------------------------------------------------ profiling --
struct PhaseScope {
    picgpu_ctx* c;
    int phase;
    cudaEvent_t a = nullptr, b = nullptr;
    PhaseScope(picgpu_ctx* c_, int ph) : c(c_), phase(ph) {
        if (!c->profiling) return;
        a = get();
        b = get();
        cudaEventRecord(a, c->stream);
    }
    cudaEvent_t get() {
        if (!c->free_events.empty()) {
            cudaEvent_t e = c->free_events.back();
            c->free_events.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    ~PhaseScope() {
        if (!c->profiling) return;
        cudaEventRecord(b, c->stream);
        c->pending.push_back({a, b, phase});
    }
};

void harvest_events(picgpu_ctx* c) {
    for (auto& ep : c->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(ep.b) == cudaSuccess && cudaEventElapsedTime(&ms, ep.a, ep.b) == cudaSuccess) {
            c->phase_ms[ep.phase] += ms;
            c->phase_launches[ep.phase] += 1;
        }
        c->free_events.push_back(ep.a);
        c->free_events.push_back(ep.b);
    }
    c->pending.clear();
}

// --------------------------------------------------------- species store --
picgpu_status alloc_species(picgpu_ctx* c, int s, long cap) {
    SpeciesBuf& b = c->sp[s];
    for (int k = 0; k < 2; ++k) {
        dfree(c, b.tet[k]);
        for (int a = 0; a < 3; ++a) {
            dfree(c, b.y64[k][a]); dfree(c, b.u64[k][a]); dfree(c, b.y32[k][a]); dfree(c, b.u32[k][a]);
            b.y64[k][a] = b.u64[k][a] = nullptr;
            b.y32[k][a] = b.u32[k][a] = nullptr;
        }
        b.tet[k] = nullptr;
        dfree(c, b.nw[k]);
        dfree(c, b.zq[k]);
        b.nw[k] = nullptr;
        b.zq[k] = nullptr;
    }
    b.cap = cap;
    b.cur = 0;
    for (int k = 0; k < 2; ++k) {
        picgpu_status st = dalloc(c, &b.tet[k], cap);
        if (st) return st;
        if (b.attrs && ((st = dalloc(c, &b.nw[k], cap)) || (st = dalloc(c, &b.zq[k], cap)))) return st;
        for (int a = 0; a < 3; ++a) {
            if (c->mixed) {
                if ((st = dalloc(c, &b.y32[k][a], cap))) return st;
                if ((st = dalloc(c, &b.u32[k][a], cap))) return st;
            } else {
                if ((st = dalloc(c, &b.y64[k][a], cap))) return st;
                if ((st = dalloc(c, &b.u64[k][a], cap))) return st;
            }
        }
    }
    return PICGPU_OK;
}

// Enlarge a species store, keeping its particles (in slot 0 of the new store).
picgpu_status grow_species(picgpu_ctx* c, int s, long cap) {
    SpeciesBuf& b = c->sp[s];
    SpeciesBuf old = b;
    const int k = old.cur;
    SpeciesBuf nb;
    nb.n = old.n;
    nb.alive = old.alive;
    nb.cap = cap;
    nb.attrs = old.attrs;
    picgpu_status st;
    for (int q = 0; q < 2; ++q) {
        if ((st = dalloc(c, &nb.tet[q], cap))) return st;
        if (nb.attrs && ((st = dalloc(c, &nb.nw[q], cap)) || (st = dalloc(c, &nb.zq[q], cap)))) return st;
        for (int a = 0; a < 3; ++a) {
            if (c->mixed) {
                if ((st = dalloc(c, &nb.y32[q][a], cap)) || (st = dalloc(c, &nb.u32[q][a], cap))) return st;
            } else {
                if ((st = dalloc(c, &nb.y64[q][a], cap)) || (st = dalloc(c, &nb.u64[q][a], cap))) return st;
            }
        }
    }
    const size_t n = size_t(old.n);
    CK(cudaMemcpyAsync(nb.tet[0], old.tet[k], n * sizeof(int32_t), cudaMemcpyDeviceToDevice, c->stream));
    if (nb.attrs) {
        CK(cudaMemcpyAsync(nb.nw[0], old.nw[k], n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(nb.zq[0], old.zq[k], n * sizeof(int32_t), cudaMemcpyDeviceToDevice, c->stream));
    }
    for (int a = 0; a < 3; ++a) {
        if (c->mixed) {
            CK(cudaMemcpyAsync(nb.y32[0][a], old.y32[k][a], n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
            CK(cudaMemcpyAsync(nb.u32[0][a], old.u32[k][a], n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
        } else {
            CK(cudaMemcpyAsync(nb.y64[0][a], old.y64[k][a], n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
            CK(cudaMemcpyAsync(nb.u64[0][a], old.u64[k][a], n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 2; ++q) {
        dfree(c, old.tet[q]);
        dfree(c, old.nw[q]);
        dfree(c, old.zq[q]);
        for (int a = 0; a < 3; ++a) {
            dfree(c, old.y64[q][a]); dfree(c, old.u64[q][a]); dfree(c, old.y32[q][a]); dfree(c, old.u32[q][a]);
        }
    }
    b = nb;
    b.cur = 0;
    return PICGPU_OK;
}

pgd::DSpecies view(const picgpu_ctx* c, int s, int k) {
    const SpeciesBuf& b = c->sp[s];
    pgd::DSpecies v{};
    v.tet = b.tet[k];
    v.nw = b.attrs ? b.nw[k] : nullptr;
    v.zq = b.attrs ? b.zq[k] : nullptr;
    for (int a = 0; a < 3; ++a) {
        v.y64[a] = b.y64[k][a];
        v.u64[a] = b.u64[k][a];
        v.y32[a] = b.y32[k][a];
        v.u32[a] = b.u32[k][a];
    }
    return v;
}

// Whether a collision model that takes its weights per species (background
// and parcel MCC, ion-neutral MCC, binary collisions) uses species s.
bool species_weight_models(const picgpu_config& cfg, int s) {
    const picgpu_mcc& m = cfg.mcc;
    const picgpu_ion_mcc& im = cfg.ion_mcc;
    if (m.enabled && (s == cfg.electron_species || (m.create_ion && s == m.ion_species) ||
                      (m.neutral_parcels && s == m.neutral_species)))
        return true;
    if (im.enabled && (s == im.ion_species || (im.neutral_parcels && s == im.neutral_species))) return true;
    if (cfg.binary.enabled && cfg.species[s].charge == 0.0) return true;
    return false;
}

// Per-parcel attributes for species s: both halves of the store get the
// arrays, the parcels stored so far the defaults (species weight, charge
// modifier 1).
picgpu_status enable_attributes(picgpu_ctx* c, int s) {
    SpeciesBuf& b = c->sp[s];
    if (b.attrs) return PICGPU_OK;
    if (species_weight_models(c->cfg, s))
        return bad(c, PICGPU_NOT_SUPPORTED,
                   "per-parcel weights: the MCC, ion-neutral and binary collision models of this library take one "
                   "weight per species");
    if (c->n_cases > 1 || !c->graphs.empty())
        return bad(c, PICGPU_NOT_SUPPORTED, "per-parcel attributes are not supported with ensembles or graph steps");
    picgpu_status st;
    if (b.cap > 0)
        for (int k = 0; k < 2; ++k)
            if ((st = dalloc(c, &b.nw[k], size_t(b.cap))) || (st = dalloc(c, &b.zq[k], size_t(b.cap)))) return st;
    b.attrs = true;
    pgd::launch_fill_attributes(view(c, s, b.cur), 0, b.n, c->cfg.species[s].weight, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return PICGPU_OK;
}

int grid_for(const picgpu_ctx* c, long n, int per_thread_block = 256) {
    const long want = (n + per_thread_block - 1) / per_thread_block;
    const long cap = long(c->sm_count) * 8;
    return int(std::max<long>(1, std::min(want, cap)));
}

pgd::MoveParams move_params(picgpu_ctx* c, int s, bool deposit_only) {
    const picgpu_species& S = c->cfg.species[s];
    pgd::MoveParams P{};
    P.m = c->dm;
    P.n = int(c->sp[s].n);
    P.species = s;
    P.pusher = c->cfg.pusher;
    P.field_weighting = c->cfg.field_weighting;
    P.charge_distribution = c->cfg.charge_distribution;
    P.deposit_mode = c->cfg.deposit_mode;
    P.rotation = c->rotation;
    P.solve_movement = deposit_only ? 0 : S.solve_movement;
    P.sync = c->cfg.sync_velocity_at_boundary;
    P.max_steps = c->cfg.track_max_steps > 0 ? c->cfg.track_max_steps : 4096;
    P.q = S.charge;
    P.mass = S.mass;
    P.value = S.charge * S.weight;
    P.weight = S.weight;
    P.dt = c->cfg.dt;
    for (int a = 0; a < 3; ++a) P.B[a] = c->cfg.B[a];
    P.fix_scale = c->fix_scale;
    P.E = c->E;
    P.Ept = c->Ept;
    P.E32 = c->E32;
    P.Ept32 = c->Ept32;
    P.cc_data = c->cc_data;
    P.vtx_data = c->vtx_data;
    P.cc_fix = c->cc_fix;
    P.vtx_fix = c->vtx_fix;
    P.qconv = c->qconv;
    P.p = view(c, s, c->sp[s].cur);
    P.counters = c->counters + s;
    P.charged = S.charge != 0.0;
    P.has_value = S.charge * S.weight != 0.0;
    P.qm_f = float(S.charge / S.mass);
    P.dt_f = float(c->cfg.dt);
    for (int a = 0; a < 3; ++a) {
        P.B_f[a] = float(c->cfg.B[a]);
        P.centre_f[a] = float(c->m.mesh_centre[a]);
    }
    P.acc9 = c->acc9 ? c->acc9 + size_t(s) * 9 * c->m.n_cells : nullptr;
    P.Ec4 = c->Ec4;
    P.t32 = c->t32;
    P.Bc = c->Bc;
    P.Bc4 = c->Bc4;
    for (const auto& pt : c->m.patches)
        if (pt.p.kind == PICGPU_PATCH_WALL || (pt.p.kind == PICGPU_PATCH_CIRCUIT && S.charge == 0.0))
            P.reflecting = 1;
    if (c->mixed && c->dm.uniform && c->xq_count) {
        // the idle double-buffer tet array holds the crossing queue
        P.cell_mover = 1;
        for (int a = 0; a < 3; ++a) {
            P.dth[a] = c->cell_dth[a];
            P.keep[a] = c->cell_keep[a];
        }
        P.xq.queue = c->sp[s].tet[1 - c->sp[s].cur];
        P.xq.count = c->xq_count;
        P.xq.start = c->xq_start;
        P.xq.capacity = c->xq_cap;
    }
    return P;
}

picgpu_status zero_accumulators(picgpu_ctx* c) {
    CK(cudaMemsetAsync(c->cc_data, 0, sizeof(double) * c->m.n_cells, c->stream));
    CK(cudaMemsetAsync(c->vtx_data, 0, sizeof(double) * c->m.n_points, c->stream));
    CK(cudaMemsetAsync(c->cc_fix, 0, sizeof(long long) * c->m.n_cells, c->stream));
    CK(cudaMemsetAsync(c->vtx_fix, 0, sizeof(long long) * c->m.n_points, c->stream));
    if (c->mixed)
        CK(cudaMemsetAsync(c->acc9, 0, sizeof(unsigned long long) * c->cfg.n_species * 9 * size_t(c->m.n_cells),
                           c->stream));
    return PICGPU_OK;
}

// Move (or deposit only) every species; counters land in c->counters.
picgpu_status move_species(picgpu_ctx* c, bool deposit_only) {
    CK(cudaMemsetAsync(c->counters, 0, sizeof(pgd::MoveCounters) * PICGPU_MAX_SPECIES, c->stream));
    for (int s = 0; s < c->cfg.n_species; ++s) {
        if (c->sp[s].n == 0) continue;
        const pgd::MoveParams P = move_params(c, s, deposit_only);
        const int grid = grid_for(c, c->sp[s].n);
        {
            PhaseScope ps(c, PICGPU_PHASE_MOVE);
            if (c->mixed) {
                c->launches += pgd::launch_move_fp32(P, 5 * c->sm_count, c->stream);
            } else {
                pgd::launch_move_fp64(P, grid, c->stream);
                c->launches++;
            }
        }
    }
    CK(cudaGetLastError());
    return PICGPU_OK;
}

picgpu_status charge_update(picgpu_ctx* c) {
    PhaseScope ps(c, PICGPU_PHASE_CHARGE);
    if (c->mixed) {
        pgd::SpeciesValues sv{};
        sv.n = c->cfg.n_species;
        for (int s = 0; s < sv.n; ++s)
            sv.v[s] = std::ldexp(c->cfg.species[s].charge * c->cfg.species[s].weight, -pgd::kDepositBits);
        const int vw = c->cfg.charge_distribution == PICGPU_WEIGHTING_VOLUME;
        pgd::launch_charge_update_mixed(c->dm, vw, sv, c->acc9, c->vtx_data, c->cfg.space_charge, c->rho,
                                        c->stream);
        c->launches += vw ? 2 : 1;
        CK(cudaGetLastError());
        return PICGPU_OK;
    }
    pgd::launch_charge_update(c->dm, c->cfg.charge_distribution == PICGPU_WEIGHTING_VOLUME,
                              c->cfg.deposit_mode == PICGPU_DEPOSIT_FIXED_POINT, c->fix_scale, c->cc_data,
                              c->vtx_data, c->cc_fix, c->vtx_fix, c->cfg.space_charge, c->rho, c->stream);
    c->launches++;
    CK(cudaGetLastError());
    return PICGPU_OK;
}

picgpu_status efield(picgpu_ctx* c) {
    PhaseScope ps(c, PICGPU_PHASE_EFIELD);
    pgd::launch_efield(c->dm, c->phi, c->grad_bc, c->E, c->Eb, c->Ept, c->E32, c->Ept32, c->stream);
    c->launches += c->dm.n_bfaces > 0 ? 4 : 3;
    if (c->Ec4) {
        pgd::launch_corner_E(c->dm, c->E, c->Ept, c->Ec4, c->stream);
        c->launches++;
    }
    CK(cudaGetLastError());
    return PICGPU_OK;
}

picgpu_status set_applied_field(picgpu_ctx* c) {
    std::vector<double> e(3 * size_t(c->m.n_cells)), ep(3 * size_t(c->m.n_points));
    for (size_t i = 0; i < e.size(); ++i) e[i] = c->cfg.E_applied[i % 3];
    for (size_t i = 0; i < ep.size(); ++i) ep[i] = c->cfg.E_applied[i % 3];
    CK(cudaMemcpyAsync(c->E, e.data(), e.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->Ept, ep.data(), ep.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    pgd::launch_to_float(c->E, c->E32, long(e.size()), c->stream);
    pgd::launch_to_float(c->Ept, c->Ept32, long(ep.size()), c->stream);
    c->launches += 2;
    if (c->Ec4) {
        pgd::launch_corner_E(c->dm, c->E, c->Ept, c->Ec4, c->stream);
        c->launches++;
    }
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

// Poisson PCG from the current phi; fills stats.
picgpu_status poisson(picgpu_ctx* c, picgpu_step_stats* stats, bool learned = false) {
    const int n = c->m.n_cells;
    const double tol = c->cfg.pcg_tol > 0 ? c->cfg.pcg_tol : 1e-10;
    const int maxit = c->cfg.pcg_max_iter > 0 ? c->cfg.pcg_max_iter : 10000;
    {
        PhaseScope ps(c, PICGPU_PHASE_POISSON);
        // PCG iterations run as a CUDA graph of kGraphIters iterations
        // (2 kernels each); iterations after convergence return at once, so
        // the iteration count stays exact.  The host checks the done flag
        // after each replay.
        if (!c->pcg_graph && !c->mg) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            for (int j = 0; j < kGraphIters; ++j)
                pgd::launch_pcg_iteration(c->dm, c->phi, c->r, c->z, c->q, c->p[0], c->p[1], c->part, c->st, maxit,
                                          c->stream);
            CK(cudaStreamEndCapture(c->stream, &g));
            CK(cudaGraphInstantiate(&c->pcg_graph, g, 0));
            CK(cudaGraphDestroy(g));
        }
        pgd::launch_rhs(c->dm, c->rho, c->grad_bc, c->b, !c->m.has_dirichlet, c->part, c->st, c->stream);
        if (learned && c->ws) {
            CK(c->ws->before(c->dm, c->b, c->phi, c->stream));
        }
        c->launches += c->m.has_dirichlet ? 1 : 3;
        if (c->mg) {
            // FP64 refinement around the FP32 multigrid-preconditioned CG
            int it = 0, outer = 0;
            double rr0 = 0, rr = 0, bb = 0;
            bool conv = false;
            const int64_t l0 = c->mg->launches;
            CK(c->mg->solve(c->dm, c->b, c->phi, tol, maxit, c->stream, &it, &outer, &rr0, &rr, &bb, &conv));
            c->mg_outer = outer;
            c->launches += c->mg->launches - l0;
            c->pcg_r0 = bb > 0 ? std::sqrt(rr0 / bb) : 0.0;
            pgd::launch_of_residual(c->dm, c->b, c->phi, c->part, c->st, c->stream);
            c->launches += 2;
            if (learned && c->ws) CK(c->ws->after(c->dm, c->phi, it, c->stream));
            CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(pgd::PcgState), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            c->st_host->iters = it;
            c->st_host->rr = rr;
            c->st_host->bb = bb;
            c->st_host->converged = conv ? 1 : 0;
        } else {
            pgd::launch_pcg_init(c->dm, c->b, c->phi, c->r, c->z, c->q, c->part, c->st, tol, c->stream);
            c->launches += 2;
            CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(pgd::PcgState), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            c->pcg_r0 = c->st_host->bb > 0 ? std::sqrt(c->st_host->rr / c->st_host->bb) : 0.0;
            int launched = 0;
            while (!c->st_host->done && launched < maxit) {
                CK(cudaGraphLaunch(c->pcg_graph, c->stream));
                launched += kGraphIters;
                c->launches += 2 * kGraphIters;
                CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(pgd::PcgState), cudaMemcpyDeviceToHost, c->stream));
                CK(cudaStreamSynchronize(c->stream));
            }
            pgd::launch_of_residual(c->dm, c->b, c->phi, c->part, c->st, c->stream);
            c->launches += 2;
            if (learned && c->ws) CK(c->ws->after(c->dm, c->phi, c->st_host->iters, c->stream));
            CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(pgd::PcgState), cudaMemcpyDeviceToHost, c->stream));
        }
    }
    picgpu_status s = efield(c);
    if (s) return s;
    CK(cudaStreamSynchronize(c->stream));
    (void)n;
    const pgd::PcgState& S = *c->st_host;
    if (stats) {
        stats->pcg_iterations = S.iters;
        stats->pcg_iterations_total += S.iters;
        stats->pcg_residual_l2 = S.bb > 0 ? std::sqrt(S.rr / S.bb) : 0.0;
        stats->pcg_residual_of = S.of_residual;
        stats->pcg_residual_initial = c->pcg_r0;
        stats->pcg_refinements = c->mg ? c->mg_outer : 0;
        if (learned && c->ws) {
            stats->learned_loss = c->ws->loss;
            stats->learned_alpha = c->ws->alpha;
            stats->learned_residual = c->ws->plain_residual;
            stats->learned_active = c->ws->active;
            stats->learned_samples = c->ws->samples;
            stats->learned_fallback = c->ws->fallback;
        }
    }
    if (!std::isfinite(S.bb) || !std::isfinite(S.rr))
        return bad(c, PICGPU_NAN_DETECTED, "Poisson: the charge density or the potential is not finite");
    if (!S.converged) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "PCG did not converge within pcg_max_iter (%d iterations, %d refinements, "
                      "relative residual %.3e)", S.iters, c->mg ? c->mg_outer : 0,
                      S.bb > 0 ? std::sqrt(S.rr / S.bb) : 0.0);
        return bad(c, PICGPU_PCG_NOT_CONVERGED, msg);
    }
    return PICGPU_OK;
}

picgpu_status solve_fields(picgpu_ctx* c, picgpu_step_stats* stats, bool learned = false) {
    if (c->cfg.maxwell_solver != PICGPU_MAXWELL_ELECTROSTATIC) return PICGPU_OK;
    return poisson(c, stats, learned);
}

picgpu_status ensure_scan(picgpu_ctx* c, long n) {
    if (c->scan_cap >= n) return PICGPU_OK;
    dfree(c, c->scan_buf);
    c->scan_cap = std::max<long>(n, 1024);
    return dalloc(c, &c->scan_buf, c->scan_cap);
}

// Drop removed particles (stable).  Removed slots (tet = -1) are skipped by
// every kernel, so the store is compacted only once they exceed 1/64 of it
// (or when forced).
picgpu_status compact(picgpu_ctx* c, bool force) {
    for (int s = 0; s < c->cfg.n_species; ++s) {
        SpeciesBuf& B = c->sp[s];
        if (B.n == 0) continue;
        const long dead = B.n - B.alive;
        if (dead == 0 || (!force && dead < std::max<long>(B.n / 64, 4096))) continue;
        const long nblk = pgd::compact_blocks(B.n);
        picgpu_status st = ensure_scan(c, nblk + 1);
        if (st) return st;
        const pgd::DSpecies src = view(c, s, B.cur), dst = view(c, s, B.cur ^ 1);
        long kept = 0;
        CK(pgd::compact_species(src, dst, B.n, c->mixed, c->scan_buf, &kept, c->stream));
        c->launches += 3;
        B.n = kept;
        B.alive = kept;
        B.cur ^= 1;
    }
    return PICGPU_OK;
}

picgpu_status read_counters(picgpu_ctx* c) {
    CK(cudaMemcpyAsync(c->counters_host, c->counters, sizeof(pgd::MoveCounters) * c->cfg.n_species,
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (c->profiling) harvest_events(c);
    return PICGPU_OK;
}

void add_counters(picgpu_ctx* c, picgpu_step_stats* stats) {
    for (int k = 0; k < c->cfg.n_species; ++k) {
        const pgd::MoveCounters& m = c->counters_host[k];
        c->sp[k].alive -= long(m.absorbed);
        if (!stats) continue;
        stats->tet_steps += (int64_t)m.tet_steps;
        stats->face_crossings += (int64_t)m.faces;
        stats->wall_hits += (int64_t)m.walls;
        stats->n_absorbed[k] += (int64_t)m.absorbed;
    }
}

void fill_counts(picgpu_ctx* c, picgpu_step_stats* stats) {
    if (!stats) return;
    for (int s = 0; s < c->cfg.n_species; ++s) stats->n_particles[s] = c->sp[s].alive;
}

// One PICCloud::evolve.
// Makes room for `add` more particles after the n used slots of species s.
picgpu_status reserve_species(picgpu_ctx* c, int s, long long add) {
    SpeciesBuf& B = c->sp[s];
    const long long need = B.n + add;
    if (need > (1LL << 31)) return bad(c, PICGPU_CAPACITY, "more than 2^31 particles of one species");
    if (need <= B.cap) return PICGPU_OK;
    const long cap = long(std::min<long long>(need + need / 4 + 1024, 1LL << 31));
    if (B.n == 0) return alloc_species(c, s, cap);
    return grow_species(c, s, cap);
}

// ParticleEmitter::emitParticle for n parcels of species sp from the patch
// of I (the RNG stream of emitter `index`), then syncVelocityAtBoundary(-0.5);
// the emitted charge comes off a floating or circuit patch.
picgpu_status emit_parcels(picgpu_ctx* c, const Injector& I, int index, int patch, int sp, long long n,
                           int model, double temperature) {
    const double dt = c->cfg.dt;
    const bool any_empty = c->m.empty[0] || c->m.empty[1] || c->m.empty[2];
    const picgpu_species& S = c->cfg.species[sp];
    picgpu_status st = reserve_species(c, sp, n);
    if (st) return st;
    SpeciesBuf& B = c->sp[sp];
    pgd::InjectParams P{};
    P.m = c->dm;
    P.seed = c->cfg.seed;
    P.step = uint32_t(c->step_index);
    P.injector = index;
    P.species = sp;
    P.model = model;
    P.constrain = any_empty;
    P.mass = S.mass;
    P.temperature = temperature;
    P.n = n;
    P.n_tri = I.n_tri;
    P.tri_cum = I.tri_cum;
    P.tri_cell = I.tri_cell;
    P.tri_tet = I.tri_tet;
    P.tri_normal = I.tri_normal;
    P.tri_fc = I.tri_fc;
    P.area = I.area;
    P.patch = patch;
    const int pk = c->m.patches[patch].p.kind;
    if (pk == PICGPU_PATCH_FLOATING || pk == PICGPU_PATCH_CIRCUIT) {
        P.qconv = c->qconv;
        P.ejected_charge = double(n) * S.charge * S.weight;
    }
    P.first = B.n;
    P.tet = B.tet[B.cur];
    for (int a = 0; a < 3; ++a) {
        P.y64[a] = B.y64[B.cur][a];
        P.u64[a] = B.u64[B.cur][a];
        P.y32[a] = B.y32[B.cur][a];
        P.u32[a] = B.u32[B.cur][a];
    }
    P.error = c->inj_err;
    pgd::launch_inject(P, c->stream);
    c->launches++;
    pgd::launch_fill_attributes(view(c, sp, B.cur), B.n, B.n + n, S.weight, c->stream);
    // syncVelocityAtBoundary(-0.5) of the new parcels (ParticleEmitter.C:401)
    if (c->cfg.sync_velocity_at_boundary && S.charge != 0.0 && c->cfg.pusher != PICGPU_PUSHER_NONE) {
        pgd::MoveParams MP = move_params(c, sp, false);
        MP.first = int(B.n);
        MP.n = int(B.n + n);
        pgd::launch_push_only(MP, c->mixed, -0.5 * dt, grid_for(c, n), c->stream);
        c->launches++;
    }
    B.n += n;
    B.alive += n;
    return PICGPU_OK;
}

// boundaryModels().injection() (PICCloud.C:1435): SimpleInjection::injection
// (SimpleInjection.C:197-240) for every injector, before the move; then the
// FreeStream models and the EmissionModels.
picgpu_status inject(picgpu_ctx* c) {
    const double dt = c->cfg.dt;
    const double t = double(c->step_index + 1) * dt;  // OpenFOAM advances the time before evolve
    for (size_t i = 0; i < c->injectors.size(); ++i) {
        Injector& I = c->injectors[i];
        if (t > I.cfg.end_time) continue;
        for (int j = 0; j < I.cfg.n_species; ++j) {
            const int sp = I.cfg.species[j];
            const picgpu_species& S = c->cfg.species[sp];
            const double np = I.cfg.frequency[j] / S.weight * dt + I.remainder[j];
            const long long n = (long long)np;
            I.remainder[j] = np - double(n);
            if (n <= 0) continue;
            picgpu_status st = emit_parcels(c, I, int(i), I.cfg.patch, sp, n, I.cfg.velocity_model,
                                            I.cfg.eV[j] * 1.602176634e-19 / 1.380649e-23);
            if (st) return st;
        }
    }
    // FreeStream::injection (FreeStream.C:126-396): counts per face on the
    // device, their scan, the total read back to size the store, the parcels
    for (size_t i = 0; i < c->freestreams.size(); ++i) {
        FsInjector& Z = c->freestreams[i];
        for (int j = 0; j < Z.cfg.n_species; ++j) {
            const int sp = Z.cfg.species[j];
            pgd::FreeStreamParams P{};
            P.m = c->dm;
            P.seed = c->cfg.seed;
            P.step = uint32_t(c->step_index);
            P.injector = int(i);
            P.species = sp;
            P.j = j;
            P.n_species = Z.F.n_species;
            P.n_faces = Z.F.n_faces;
            P.cell = Z.cell;
            P.tet0 = Z.tet0;
            P.frac0 = Z.frac0;
            P.n_in = Z.n_in;
            P.t1 = Z.t1;
            P.t2 = Z.t2;
            P.add = Z.add;
            P.s = Z.s;
            P.c_mp = Z.F.c_mp[j];
            P.v_t = Z.F.v_t[j];
            for (int a = 0; a < 3; ++a) P.U[a] = Z.cfg.velocity[a];
            P.acc = Z.acc;
            P.counts = Z.counts;
            P.offsets = Z.offsets;
            P.error = c->inj_err;
            pgd::launch_freestream_count(P, c->stream);
            CK(pgd::init_scan(Z.counts, Z.offsets, Z.sums, Z.F.n_faces, c->stream));
            long long total = 0;
            CK(cudaMemcpyAsync(&total, Z.offsets + Z.F.n_faces, sizeof total, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            c->launches += 4;
            if (total <= 0) continue;
            picgpu_status st = reserve_species(c, sp, total);
            if (st) return st;
            SpeciesBuf& B = c->sp[sp];
            P.first = B.n;
            P.tet = B.tet[B.cur];
            for (int a = 0; a < 3; ++a) {
                P.y64[a] = B.y64[B.cur][a];
                P.u64[a] = B.u64[B.cur][a];
                P.y32[a] = B.y32[B.cur][a];
                P.u32[a] = B.u32[B.cur][a];
            }
            pgd::launch_freestream_emit(P, c->stream);
            c->launches++;
            // syncVelocityAtBoundary(-0.5) of the new parcels (FreeStream.C:385)
            const picgpu_species& S = c->cfg.species[sp];
            pgd::launch_fill_attributes(view(c, sp, B.cur), B.n, B.n + total, S.weight, c->stream);
            if (c->cfg.sync_velocity_at_boundary && S.charge != 0.0 && c->cfg.pusher != PICGPU_PUSHER_NONE) {
                pgd::MoveParams MP = move_params(c, sp, false);
                MP.first = int(B.n);
                MP.n = int(B.n + total);
                pgd::launch_push_only(MP, c->mixed, -0.5 * c->cfg.dt, grid_for(c, total), c->stream);
                c->launches++;
            }
            B.n += total;
            B.alive += total;
        }
    }
    // EmissionModels (SM/Helper/Emission): n = J A dt / (w e) + remainder
    for (size_t i = 0; i < c->emitters.size(); ++i) {
        Injector& I = c->emitters[i];
        const int sp = c->cfg.electron_species;
        const picgpu_species& S = c->cfg.species[sp];
        const double qe = std::fabs(S.charge);
        double j = I.em_j;
        double temperature = I.em.temperature;
        if (I.em.model == PICGPU_EMISSION_FOWLER_NORDHEIM) {
            pgd::launch_fowler_nordheim(c->dm, c->Eb, I.em_faces, I.em_n_faces, I.em.work_function, c->em_sum,
                                        c->stream);
            c->launches++;
            CK(cudaMemcpyAsync(&j, c->em_sum, sizeof j, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            temperature = I.em.work_function * qe / 1.380649e-23;
        }
        const double ne = j * I.area * dt / (S.weight * qe) + I.em_remainder;
        const long long n = (long long)ne;
        I.em_remainder = ne - double(n);
        if (n <= 0) continue;
        picgpu_status st = emit_parcels(c, I, PICGPU_MAX_INJECTORS + int(i), I.em.patch, sp, n,
                                        PICGPU_EMIT_MAXWELLIAN_FLUX, temperature);
        if (st) return st;
    }
    CK(cudaGetLastError());
    return PICGPU_OK;
}

// PairMerging over the listed species, in list order: each species' merges
// are selected on its occupancy (slots [0, n_occ)), then the merged parcels
// appended behind the store.
picgpu_status merge_parcels(picgpu_ctx* c, picgpu_step_stats* stats, const long* n_occ) {
    const picgpu_merging& mg = c->cfg.merging;
    pgd::CollideArgs a{};
    a.m = c->dm;
    a.cfg = &c->cfg;
    a.step = c->step_index;
    a.n_species = c->cfg.n_species;
    a.mixed = c->mixed;
    a.stream = c->stream;
    std::string msg;
    for (int li = 0; li < mg.n_species; ++li) {
        const int sp = mg.species[li];
        SpeciesBuf& B = c->sp[sp];
        a.sp[sp] = view(c, sp, B.cur);
        a.n[sp] = std::min(n_occ[sp], B.n);
        a.cap[sp] = B.cap;
        long long total = 0;
        int e = pgd::merge_select(c->coll, a, li, sp, &total, &msg, &c->launches);
        if (e) return bad(c, picgpu_status(e), msg);
        if (total <= 0) continue;
        picgpu_status st = reserve_species(c, sp, total);
        if (st) return st;
        a.sp[sp] = view(c, sp, B.cur);
        e = pgd::merge_append(c->coll, a, sp, B.n, total, &msg, &c->launches);
        if (e) return bad(c, picgpu_status(e), msg);
        B.n += total;
        B.alive -= total;   // two parcels out, one in, per merge
    }
    long long merged = 0, checked = 0;
    double kin = 0.0;
    if (pgd::merge_counters(c->coll, c->stream, &merged, &checked, &kin)) CK(cudaGetLastError());
    if (stats) {
        stats->merged_parcels += merged;
        stats->merge_checks += checked;
        stats->merge_kinetic_energy_error += kin;
    }
    return PICGPU_OK;
}

picgpu_status one_step(picgpu_ctx* c, picgpu_step_stats* stats, bool fields) {
    picgpu_status s;
    if ((!c->injectors.empty() || !c->freestreams.empty() || !c->emitters.empty()) && (s = inject(c))) return s;
    if ((s = zero_accumulators(c))) return s;
    if ((s = move_species(c, false))) return s;
    // Without collisions the charge update needs nothing the host decides
    // from the move counters (it reads the deposit accumulators only), so it
    // is queued before the counters are read: one wait per step.
    const bool colliding = c->cfg.mcc.enabled || c->cfg.coulomb.enabled || c->cfg.ion_mcc.enabled ||
                           c->cfg.binary.enabled;
    if (!colliding) {
        CK(cudaMemcpyAsync(c->counters_host, c->counters, sizeof(pgd::MoveCounters) * c->cfg.n_species,
                           cudaMemcpyDeviceToHost, c->stream));
        if ((s = charge_update(c))) return s;
        CK(cudaStreamSynchronize(c->stream));
        if (c->profiling) harvest_events(c);
    } else if ((s = read_counters(c))) {
        return s;
    }
    int err = 0;
    for (int k = 0; k < c->cfg.n_species; ++k) err = std::max(err, c->counters_host[k].error);
    if (err)
        return bad(c, picgpu_status(err), err == PICGPU_SPEED_OF_LIGHT
                                              ? "particle velocity reached the speed of light"
                                              : "tracking exceeded track_max_steps for a particle");
    add_counters(c, stats);
    if (!c->injectors.empty() || !c->freestreams.empty() || !c->emitters.empty()) {
        int ie = 0;
        CK(cudaMemcpy(&ie, c->inj_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (ie == 2) return bad(c, PICGPU_INVALID_ARG, "freestream: more than 2^30 parcels on one face in one step");
        if (ie) return bad(c, PICGPU_INVALID_ARG, "injection: an emitted parcel left its owner cell");
    }
    if (c->cfg.sort_interval > 0 && (c->step_index + 1) % c->cfg.sort_interval == 0) {
        // cell re-sort (keeps each block's particles in a short cell range)
        PhaseScope ps(c, PICGPU_PHASE_SORT);
        for (int k = 0; k < c->cfg.n_species; ++k) {
            SpeciesBuf& B = c->sp[k];
            if (B.n == 0) continue;
            long kept = 0;
            std::string msg;
            const int e = pgd::sort_species(c->coll, c->dm, k, view(c, k, B.cur), view(c, k, B.cur ^ 1), B.n,
                                            c->mixed, &kept, c->stream, &msg, &c->launches);
            if (e) return bad(c, picgpu_status(e), msg);
            B.n = kept;
            B.alive = kept;
            B.cur ^= 1;
        }
    } else if ((s = compact(c, false))) {
        return s;
    }
    // the parcels of the cell occupancy (PICCloud::buildCellOccupancy):
    // collision secondaries of this step come after them
    long n_occ[PICGPU_MAX_SPECIES] = {};
    for (int k = 0; k < c->cfg.n_species; ++k) n_occ[k] = c->sp[k].n;
    if (colliding) {
        if ((s = pgd_collisions(c, stats))) return s;
        if ((s = charge_update(c))) return s;
    }
    if (!fields) return PICGPU_OK;
    pgd::launch_floating_update(c->qconv, c->sigma, c->grad_bc, c->stream);
    c->launches++;
    // circuit models around the field solve (PICCloud.C:1457-1464); the
    // source and the averaging factor are evaluated here, on the host
    const double t_now = double(c->step_index + 1) * c->cfg.dt;
    const double src = c->circ.model == PICGPU_CIRCUIT_RLC ? pg::circuit_source(c->cfg.circuit, t_now) : 0.0;
    if (c->circ.model != PICGPU_CIRCUIT_NONE) {
        pgd::launch_circuit_pre(c->circ, src, c->qconv, c->grad_bc, c->circ_state, c->stream);
        c->launches++;
    }
    if ((s = solve_fields(c, stats, true))) return s;
    if (c->circ.model != PICGPU_CIRCUIT_NONE) {
        pgd::launch_circuit_post(c->circ, c->dm, src, c->cfg.dt / t_now, c->phi, c->qconv, c->circ_state,
                                 c->stream);
        c->launches++;
    }
    // ParticleMerging::checkAndMerge, the last call of the step (PICCloud.C:1470)
    if (c->cfg.merging.enabled && (s = merge_parcels(c, stats, n_occ))) return s;
    c->step_index++;
    return PICGPU_OK;
}

}  // namespace

// Collisions live in collide.cu; this bridge keeps the context private.
picgpu_status pgd_collisions(picgpu_ctx* c, picgpu_step_stats* stats) {
    // room for MCC secondaries: at least an eighth of the population free
    for (int s = 0; s < c->cfg.n_species; ++s) {
        const long need = c->sp[s].n + std::max<long>(c->sp[s].n / 8, 4096);
        if (need > c->sp[s].cap) {
            const picgpu_status g = grow_species(c, s, need + need / 2);
            if (g) return g;
        }
    }
    pgd::CollideArgs a{};
    a.m = c->dm;
    a.cfg = &c->cfg;
    a.step = c->step_index;
    a.n_species = c->cfg.n_species;
    a.mixed = c->mixed;
    for (int s = 0; s < c->cfg.n_species; ++s) {
        a.sp[s] = view(c, s, c->sp[s].cur);
        a.n[s] = c->sp[s].n;
        a.cap[s] = c->sp[s].cap;
    }
    a.stream = c->stream;
    int64_t counts[pgd::kCollideCounts] = {};
    long newn[PICGPU_MAX_SPECIES] = {};
    int swapped[PICGPU_MAX_SPECIES] = {};
    std::string msg;
    picgpu_status st;
    {
        PhaseScope ps(c, c->cfg.mcc.enabled ? PICGPU_PHASE_MCC : PICGPU_PHASE_COULOMB);
        st = picgpu_status(pgd::run_collisions(c->coll, a, counts, newn, swapped, &msg, &c->launches, nullptr));
    }
    if (st) return bad(c, st, msg);
    // neutral parcels deleted by ionisation stay in the store as removed slots
    if (c->cfg.mcc.enabled && c->cfg.mcc.neutral_parcels) c->sp[c->cfg.mcc.neutral_species].alive -= counts[12];
    for (int s = 0; s < c->cfg.n_species; ++s) {
        const long old = c->sp[s].n;
        c->sp[s].n = newn[s];
        c->sp[s].alive += newn[s] - old;
        if (newn[s] > old) {
            // parcels created by the MCC models carry the species defaults
            // (PICCloud::addNewParcel, PICCloud.C:707-723); the electrons of
            // Perez ionisations, appended first, have their own nParticle
            const long own = s == c->cfg.electron_species ? long(counts[21]) : 0;
            pgd::launch_fill_attributes(view(c, s, c->sp[s].cur), old + own, newn[s], c->cfg.species[s].weight,
                                        c->stream);
            // deposit the secondaries created this step (calculateFields sees
            // every parcel, PICCloud.C:616-660)
            pgd::MoveParams P = move_params(c, s, true);
            P.first = int(old);
            if (c->mixed) {
                c->launches += pgd::launch_move_fp32(P, 5 * c->sm_count, c->stream);
            } else {
                pgd::launch_move_fp64(P, grid_for(c, newn[s] - old), c->stream);
                c->launches++;
            }
        }
    }
    CK(cudaGetLastError());
    if (stats) {
        stats->mcc_candidates += counts[0];
        stats->mcc_elastic += counts[1];
        stats->mcc_excitation += counts[2];
        stats->mcc_ionization += counts[3];
        stats->coulomb_pairs += counts[4];
        stats->coulomb_ionizations += counts[20];
        stats->coulomb_ionization_electrons += counts[21];
        stats->ion_mcc_candidates += counts[5];
        stats->ion_mcc_elastic += counts[6];
        stats->ion_mcc_charge_exchange += counts[7];
        stats->binary_candidates += counts[8];
        stats->binary_collisions += counts[9];
        stats->binary_background_candidates += counts[10];
        stats->binary_background_collisions += counts[11];
        stats->mcc_parcel_candidates += counts[pgd::kCountMccParcel];
        stats->mcc_parcel_elastic += counts[pgd::kCountMccParcel + 1];
        stats->mcc_parcel_excitation += counts[pgd::kCountMccParcel + 2];
        stats->mcc_parcel_ionization += counts[pgd::kCountMccParcel + 3];
        stats->ion_parcel_candidates += counts[pgd::kCountIonParcel];
        stats->ion_parcel_elastic += counts[pgd::kCountIonParcel + 1];
        stats->ion_parcel_charge_exchange += counts[pgd::kCountIonParcel + 2];
    }
    return PICGPU_OK;
}

namespace {

// ------------------------------------------------- graph-stepped runs --
__global__ void step_inc_kernel(unsigned* step) { *step += 1u; }

// Per case and species: count, sum U, sum |U|^2 (shared-memory partials).
template <class R>
__global__ void case_stats_kernel(const int32_t* __restrict__ tet, const R* __restrict__ u0,
                                  const R* __restrict__ u1, const R* __restrict__ u2, long n, int cells_per_case,
                                  int n_cases, double* __restrict__ out) {
    extern __shared__ double sh[];  // n_cases * 5
    for (int k = threadIdx.x; k < n_cases * 5; k += blockDim.x) sh[k] = 0.0;
    __syncthreads();
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const int t = tet[i];
        if (t < 0) continue;
        const int k = (t / 12) / cells_per_case;
        const double a = u0[i], b = u1[i], c = u2[i];
        atomicAdd(sh + 5 * k, 1.0);
        atomicAdd(sh + 5 * k + 1, a);
        atomicAdd(sh + 5 * k + 2, b);
        atomicAdd(sh + 5 * k + 3, c);
        atomicAdd(sh + 5 * k + 4, a * a + b * b + c * c);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n_cases * 5; k += blockDim.x)
        if (sh[k] != 0.0) atomicAdd(out + k, sh[k]);
}

__global__ void case_sum_kernel(const unsigned long long* __restrict__ per_cell, int cells_per_case,
                                unsigned long long* __restrict__ out) {
    __shared__ unsigned long long s[256];
    unsigned long long v = 0;
    const size_t base = size_t(blockIdx.x) * cells_per_case;
    for (int c = threadIdx.x; c < cells_per_case; c += 256) v += per_cell[base + c];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

long total_particles(const picgpu_ctx* c) {
    long n = 0;
    for (int k = 0; k < c->cfg.n_species; ++k) n += c->sp[k].alive;
    return n;
}

bool any_collisions(const picgpu_ctx* c) {
    return c->cfg.mcc.enabled || c->cfg.coulomb.enabled || c->cfg.ion_mcc.enabled || c->cfg.binary.enabled;
}

pgd::CollideArgs collide_args(picgpu_ctx* c) {
    pgd::CollideArgs a{};
    a.m = c->dm;
    a.cfg = &c->cfg;
    a.step = c->step_index;
    a.n_species = c->cfg.n_species;
    a.mixed = c->mixed;
    for (int s = 0; s < c->cfg.n_species; ++s) {
        a.sp[s] = view(c, s, c->sp[s].cur);
        a.n[s] = c->sp[s].n;
        a.cap[s] = c->sp[s].cap;
    }
    a.stream = c->stream;
    return a;
}

// The kernels of one step with every count on the device (captured).
picgpu_status graph_step_body(picgpu_ctx* c) {
    picgpu_status s;
    if ((s = zero_accumulators(c))) return s;
    const int grid = c->move_bps * c->sm_count;
    for (int k = 0; k < c->cfg.n_species; ++k) {
        pgd::MoveParams P = move_params(c, k, false);
        P.n_dev = c->n_dev + k;
        P.first_dev = nullptr;
        c->launches += pgd::launch_move_fp32(P, grid, c->stream);
    }
    if (any_collisions(c)) {
        std::string msg;
        const pgd::CollideArgs a = collide_args(c);
        const int e = pgd::run_collisions_device(c->coll, a, c->n_dev, c->first_dev, c->step_dev, &msg, &c->launches);
        if (e) return bad(c, picgpu_status(e), msg);
        // deposit the secondaries of this step (first_dev .. n_dev)
        for (int k = 0; k < c->cfg.n_species; ++k) {
            pgd::MoveParams P = move_params(c, k, true);
            P.n_dev = c->n_dev + k;
            P.first_dev = c->first_dev + k;
            c->launches += pgd::launch_move_fp32(P, grid, c->stream);
        }
    }
    if ((s = charge_update(c))) return s;
    step_inc_kernel<<<1, 1, 0, c->stream>>>(c->step_dev);
    c->launches++;
    CK(cudaGetLastError());
    return PICGPU_OK;
}

// The graph for the current buffers and launch shapes, captured on demand.
picgpu_status graph_for(picgpu_ctx* c, int steps, cudaGraphExec_t* out) {
    uint64_t key = uint64_t(steps) | (uint64_t(c->move_bps) << 16) | (uint64_t(c->coll.mcc_block) << 24);
    for (int k = 0; k < c->cfg.n_species; ++k) key |= uint64_t(c->sp[k].cur) << (40 + k);
    for (const auto& g : c->graphs)
        if (g.key == key) {
            *out = g.exec;
            return PICGPU_OK;
        }
    cudaGraph_t g;
    // phase events are host-side bookkeeping: keep them out of the capture
    const bool prof = c->profiling;
    c->profiling = false;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    picgpu_status s = PICGPU_OK;
    for (int j = 0; j < steps && !s; ++j) s = graph_step_body(c);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->profiling = prof;
    if (s) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return s;
    }
    CK(e);
    cudaGraphExec_t exec;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    c->graphs.push_back({key, exec});
    *out = exec;
    return PICGPU_OK;
}

void drop_graphs(picgpu_ctx* c) {
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

// FNV-1a over every device pointer a captured step addresses: a graph is
// reused only while none of them moved.
uint64_t buffers_signature(const picgpu_ctx* c) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* p) {
        uint64_t v = uint64_t(reinterpret_cast<uintptr_t>(p));
        for (int i = 0; i < 8; ++i) {
            h ^= (v >> (8 * i)) & 0xFFu;
            h *= 1099511628211ull;
        }
    };
    for (int k = 0; k < c->cfg.n_species; ++k) {
        const SpeciesBuf& B = c->sp[k];
        for (int q = 0; q < 2; ++q) {
            mix(B.tet[q]);
            for (int a = 0; a < 3; ++a) {
                mix(B.y32[q][a]);
                mix(B.u32[q][a]);
            }
        }
        mix(c->coll.idx[k]);
        mix(c->coll.sel[k]);
        mix(c->coll.sel2[k]);
    }
    const void* ps[] = {c->coll.stage, c->coll.flags, c->coll.pos, c->coll.stage_tmp, c->coll.cell_start,
                        c->coll.cell_count, c->coll.cell_cursor, c->coll.scan_tmp, c->coll.ncand, c->coll.cand_off,
                        c->acc9, c->Ec4};
    for (const void* p : ps) mix(p);
    return h;
}

// Between replays: re-sort or compact, and reserve room for the next replay.
picgpu_status graph_maintenance(picgpu_ctx* c, int steps) {
    picgpu_status s;
    if (c->cfg.sort_interval > 0 && c->step_index - c->last_sort >= c->cfg.sort_interval) {
        PhaseScope ps(c, PICGPU_PHASE_SORT);
        for (int k = 0; k < c->cfg.n_species; ++k) {
            SpeciesBuf& B = c->sp[k];
            if (B.n == 0) continue;
            long kept = 0;
            std::string msg;
            const int e = pgd::sort_species(c->coll, c->dm, k, view(c, k, B.cur), view(c, k, B.cur ^ 1), B.n,
                                            c->mixed, &kept, c->stream, &msg, &c->launches);
            if (e) return bad(c, picgpu_status(e), msg);
            B.n = kept;
            B.alive = kept;
            B.cur ^= 1;
        }
        c->last_sort = c->step_index;
    } else if ((s = compact(c, false))) {
        return s;
    }
    for (int k = 0; k < c->cfg.n_species; ++k) {
        // MCC secondaries of the coming replay: keep an eighth (and per step
        // at least 1/64) of the population free
        const long n = c->sp[k].n;
        const long need = n + std::max<long>(n / 8, 4096) + long(steps) * (n / 64 + 1024);
        if (need > c->sp[k].cap && (s = grow_species(c, k, need + need / 2))) return s;
    }
    if (any_collisions(c)) {
        std::string msg;
        const pgd::CollideArgs a = collide_args(c);
        const int e = pgd::collide_reserve_device(c->coll, a, &msg);
        if (e) return bad(c, picgpu_status(e), msg);
    }
    const uint64_t sig = buffers_signature(c);
    if (sig != c->graph_sig) {
        drop_graphs(c);
        c->graph_sig = sig;
    }
    return PICGPU_OK;
}

// One replay of `steps` steps; counters accumulate into stats.
picgpu_status graph_replay(picgpu_ctx* c, int steps, picgpu_step_stats* stats, float* ms) {
    picgpu_status s;
    if ((s = graph_maintenance(c, steps))) return s;
    int nh[PICGPU_MAX_SPECIES] = {};
    for (int k = 0; k < c->cfg.n_species; ++k) nh[k] = int(c->sp[k].n);
    const unsigned step0 = unsigned(c->step_index);
    CK(cudaMemcpyAsync(c->n_dev, nh, sizeof nh, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->step_dev, &step0, sizeof step0, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->counters, 0, sizeof(pgd::MoveCounters) * PICGPU_MAX_SPECIES, c->stream));
    if (any_collisions(c)) {
        CK(cudaMemsetAsync(c->coll.counts, 0, pgd::kCollideCounts * sizeof(unsigned long long), c->stream));
        CK(cudaMemsetAsync(c->coll.overflow, 0, sizeof(int), c->stream));
    }
    cudaGraphExec_t g;
    if ((s = graph_for(c, steps, &g))) return s;
    if (!c->replay_ev[0]) {
        CK(cudaEventCreate(&c->replay_ev[0]));
        CK(cudaEventCreate(&c->replay_ev[1]));
    }
    {
        PhaseScope ps(c, PICGPU_PHASE_MOVE);
        CK(cudaEventRecord(c->replay_ev[0], c->stream));
        CK(cudaGraphLaunch(g, c->stream));
        CK(cudaEventRecord(c->replay_ev[1], c->stream));
    }
    if ((s = read_counters(c))) return s;
    int nd[PICGPU_MAX_SPECIES] = {};
    int ovf = 0;
    unsigned long long h[pgd::kCollideCounts] = {};
    CK(cudaMemcpyAsync(nd, c->n_dev, sizeof nd, cudaMemcpyDeviceToHost, c->stream));
    if (any_collisions(c)) {
        CK(cudaMemcpyAsync(&ovf, c->coll.overflow, sizeof ovf, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(h, c->coll.counts, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    if (ms) CK(cudaEventElapsedTime(ms, c->replay_ev[0], c->replay_ev[1]));
    int err = 0;
    for (int k = 0; k < c->cfg.n_species; ++k) err = std::max(err, c->counters_host[k].error);
    if (err)
        return bad(c, picgpu_status(err), err == PICGPU_SPEED_OF_LIGHT
                                              ? "particle velocity reached the speed of light"
                                              : "tracking exceeded track_max_steps for a particle");
    if (ovf) return bad(c, PICGPU_CAPACITY, "graph step: MCC staging or particle storage ran out of room");
    add_counters(c, stats);
    for (int k = 0; k < c->cfg.n_species; ++k) {
        c->sp[k].alive += long(nd[k]) - c->sp[k].n;
        c->sp[k].n = nd[k];
    }
    if (stats) {
        stats->mcc_candidates += (int64_t)h[0];
        stats->mcc_elastic += (int64_t)h[1];
        stats->mcc_excitation += (int64_t)h[2];
        stats->mcc_ionization += (int64_t)h[3];
        stats->coulomb_pairs += (int64_t)h[4];
        stats->ion_mcc_candidates += (int64_t)h[5];
        stats->ion_mcc_elastic += (int64_t)h[6];
        stats->ion_mcc_charge_exchange += (int64_t)h[7];
        stats->binary_candidates += (int64_t)h[8];
        stats->binary_collisions += (int64_t)h[9];
        stats->binary_background_candidates += (int64_t)h[10];
        stats->binary_background_collisions += (int64_t)h[11];
    }
    c->step_index += steps;
    return PICGPU_OK;
}

}  // namespace

extern "C" {

picgpu_status picgpu_mesh_create(const picgpu_mesh_desc* desc, picgpu_mesh** out) {
    if (!desc || !out) return PICGPU_INVALID_ARG;
    *out = nullptr;
    try {
        auto* m = new picgpu_mesh();
        m->m = pg::build_hex_mesh(*desc);
        *out = m;
    } catch (const std::exception&) {
        return PICGPU_INVALID_ARG;
    }
    return PICGPU_OK;
}

void picgpu_mesh_destroy(picgpu_mesh* mesh) { delete mesh; }

picgpu_status picgpu_mesh_info_get(const picgpu_mesh* mesh, picgpu_mesh_info* info) {
    if (!mesh || !info) return PICGPU_INVALID_ARG;
    info->n_cells = mesh->m.n_cells;
    info->n_points = mesh->m.n_points;
    info->n_tets = 12LL * mesh->m.n_cells;
    info->n_patches = (int64_t)mesh->m.patches.size();
    return PICGPU_OK;
}

picgpu_status picgpu_mesh_locate(const picgpu_mesh* mesh, size_t n, const double* xyz, int32_t* tet,
                                 double* bary) {
    if (!mesh || (n && (!xyz || !tet || !bary))) return PICGPU_INVALID_ARG;
    for (size_t i = 0; i < n; ++i) tet[i] = int32_t(pg::locate(mesh->m, xyz + 3 * i, bary + 3 * i));
    return PICGPU_OK;
}

picgpu_status picgpu_mesh_position(const picgpu_mesh* mesh, size_t n, const int32_t* tet, const double* bary,
                                   double* xyz) {
    if (!mesh || (n && (!xyz || !tet || !bary))) return PICGPU_INVALID_ARG;
    const long long nt = 12LL * mesh->m.n_cells;
    for (size_t i = 0; i < n; ++i) {
        if (tet[i] < 0 || tet[i] >= nt) return PICGPU_INVALID_ARG;
        pg::position(mesh->m, tet[i], bary + 3 * i, xyz + 3 * i);
    }
    return PICGPU_OK;
}

picgpu_status picgpu_mesh_cells(const picgpu_mesh* mesh, double* centres, double* volumes) {
    if (!mesh) return PICGPU_INVALID_ARG;
    if (centres) std::memcpy(centres, mesh->m.cc.data(), mesh->m.cc.size() * sizeof(double));
    if (volumes) std::memcpy(volumes, mesh->m.vol.data(), mesh->m.vol.size() * sizeof(double));
    return PICGPU_OK;
}

static picgpu_status create_with_mesh(picgpu_ctx* c, const picgpu_config* cfg);

// Device staging of row-major host arrays (n tets, n x 3 bary, n x 3 U).
static picgpu_status ensure_rows(picgpu_ctx* c, size_t n) {
    if (c->rows_cap >= n) return PICGPU_OK;
    dfree(c, c->rows_tet);
    dfree(c, c->rows_y);
    dfree(c, c->rows_u);
    c->rows_cap = 0;
    const size_t cap = std::max<size_t>(n, 1024);
    picgpu_status s;
    if ((s = dalloc(c, &c->rows_tet, cap)) || (s = dalloc(c, &c->rows_y, 3 * cap)) ||
        (s = dalloc(c, &c->rows_u, 3 * cap)))
        return s;
    c->rows_cap = cap;
    return PICGPU_OK;
}

picgpu_status picgpu_create(const picgpu_mesh_desc* mesh, const picgpu_config* cfg, picgpu_ctx** out) {
    if (!mesh || !cfg || !out) return PICGPU_INVALID_ARG;
    auto* c = new picgpu_ctx();
    *out = c;
    try {
        c->m = pg::build_hex_mesh(*mesh);
    } catch (const std::exception& e) {
        return bad(c, PICGPU_INVALID_ARG, e.what());
    }
    return create_with_mesh(c, cfg);
}

picgpu_status picgpu_ensemble_create(const picgpu_mesh_desc* one_case, int n_cases, const picgpu_config* cfg,
                                     picgpu_ctx** out) {
    if (!one_case || !cfg || !out || n_cases < 1) return PICGPU_INVALID_ARG;
    auto* c = new picgpu_ctx();
    *out = c;
    try {
        const pg::HexMesh one = pg::build_hex_mesh(*one_case);
        if (long(one.n_cells) * n_cases > (1L << 31) / 12 - 1)
            return bad(c, PICGPU_INVALID_ARG, "ensemble: too many cells for 32-bit tet indices");
        c->m = pg::replicate_mesh(one, n_cases);
    } catch (const std::exception& e) {
        return bad(c, PICGPU_INVALID_ARG, e.what());
    }
    c->n_cases = n_cases;
    return create_with_mesh(c, cfg);
}

static picgpu_status create_with_mesh(picgpu_ctx* c, const picgpu_config* cfg) {
    if (cfg->n_species < 1 || cfg->n_species > PICGPU_MAX_SPECIES)
        return bad(c, PICGPU_INVALID_ARG, "config: n_species must be 1..4");
    if (!(cfg->dt > 0)) return bad(c, PICGPU_INVALID_ARG, "config: dt must be > 0");
    if (cfg->pusher < PICGPU_PUSHER_NONE || cfg->pusher > PICGPU_PUSHER_HIGUERA_CARY)
        return bad(c, PICGPU_INVALID_ARG, "config: unknown ParticlePusher");
    if (cfg->precision != PICGPU_PREC_FP64 && cfg->precision != PICGPU_PREC_MIXED)
        return bad(c, PICGPU_INVALID_ARG, "config: unknown precision");
    if (cfg->pcg_precond != PICGPU_PRECOND_JACOBI && cfg->pcg_precond != PICGPU_PRECOND_MULTIGRID)
        return bad(c, PICGPU_INVALID_ARG, "config: unknown PCG preconditioner");
    {
        const std::string ce = pg::check_circuit(c->m, cfg->circuit, cfg->dt);
        if (!ce.empty()) return bad(c, PICGPU_INVALID_ARG, ce);
        if (cfg->circuit.model != PICGPU_CIRCUIT_NONE && c->n_cases > 1)
            return bad(c, PICGPU_NOT_SUPPORTED, "circuit: not for ensemble contexts");
    }
    c->cfg = *cfg;
    c->mixed = cfg->precision == PICGPU_PREC_MIXED;
    c->rotation = cfg->B[0] != 0.0 || cfg->B[1] != 0.0 || cfg->B[2] != 0.0;
    double qmax = 0;
    for (int s = 0; s < cfg->n_species; ++s)
        qmax = std::fmax(qmax, std::fabs(cfg->species[s].charge * cfg->species[s].weight));
    c->fix_scale = qmax > 0 ? std::ldexp(1.0, 39 - std::ilogb(qmax)) : 1.0;

    CK(cudaGetDevice(&c->device));
    CK(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device));
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));

    const pg::HexMesh& m = c->m;
    // tables
    for (int t = 0; t < 12; ++t) {
        for (int j = 0; j < 3; ++j) c->tc.tri[t][j] = int8_t(m.tt.tri[t][j]);
        for (int i = 0; i < 4; ++i) {
            c->tc.inner_next[t][i] = int8_t(m.tt.inner_next[t][i]);
            for (int j = 0; j < 4; ++j) c->tc.inner_src[t][i][j] = int8_t(m.tt.inner_src[t][i][j]);
        }
        c->tc.cross_next[t] = int8_t(m.tt.cross_next[t]);
        for (int j = 0; j < 4; ++j) c->tc.cross_src[t][j] = int8_t(m.tt.cross_src[t][j]);
    }
    if (m.patches.size() > size_t(pgd::kMaxPatches)) return bad(c, PICGPU_INVALID_ARG, "too many patches");
    c->pc.n = int(m.patches.size());
    for (size_t p = 0; p < m.patches.size(); ++p) {
        c->pc.kind[p] = m.patches[p].p.kind;
        c->pc.phi_bc[p] = m.patches[p].p.phi_bc;
        c->pc.phi[p] = m.patches[p].p.phi;
        c->pc.area[p] = m.patches[p].area;
        c->pc.rlc_k[p] = 0.0;
    }
    if (cfg->circuit.model != PICGPU_CIRCUIT_NONE) {
        const picgpu_circuit& cc = cfg->circuit;
        const double area = m.patches[cc.cathode_patch].area;
        const pg::RlcCoeffs rc = pg::rlc_coefficients(cc, cfg->dt, area);
        pgd::CircuitParams& P = c->circ;
        P.model = cc.model;
        P.anode = cc.anode_patch;
        P.cathode = cc.cathode_patch;
        for (int i = 0; i < 5; ++i) P.a[i] = rc.a[i];
        P.k = rc.k;
        P.area = area;
        P.I = pg::circuit_current_source(cc, area);
        P.dt = cfg->dt;
        if (cc.model == PICGPU_CIRCUIT_RLC) c->pc.rlc_k[cc.cathode_patch] = rc.k;
    }
    CK(pgd::move_fp64_set_tables(c->tc, c->pc));
    CK(pgd::init_set_tables(c->tc));
    {
        std::vector<double> tv(12 * size_t(std::max(m.n_classes, 1)), 0.0);
        for (int k = 0; k < m.n_classes; ++k)
            for (int t = 0; t < 12; ++t) tv[12 * size_t(k) + t] = pg::tet_volume(m, k, t);
        const picgpu_status us = upload(c, &c->tet_vol, tv);
        if (us) return us;
    }
    {
        // FP32 kernel tables: class-0 geometry (used when the mesh has one
        // class) and the packed crossing codes
        pgd::Tables32 t{};
        for (int k = 0; k < 108; ++k) t.inv[k] = float(m.cls_tetinv[k]);
        for (int k = 0; k < 18; ++k) t.normal[k] = float(m.cls_fnormal[k]);
        for (int k = 0; k < 24; ++k) t.off[k] = float(m.cls_offset[k]);
        auto enc = [](int nt, const int* src) {
            unsigned code = unsigned(nt);
            for (int j = 0; j < 4; ++j) code |= unsigned(src[j] < 0 ? 7 : src[j]) << (4 + 3 * j);
            return code;
        };
        for (int tt = 0; tt < 12; ++tt) {
            for (int i = 1; i < 4; ++i) t.inner[4 * tt + i] = enc(m.tt.inner_next[tt][i], m.tt.inner_src[tt][i]);
            t.cross[tt] = enc(m.tt.cross_next[tt], m.tt.cross_src[tt]);
            t.tri[tt] = unsigned(m.tt.tri[tt][0]) | unsigned(m.tt.tri[tt][1]) << 4 | unsigned(m.tt.tri[tt][2]) << 8;
        }
        for (size_t p = 0; p < m.patches.size(); ++p) t.kind[p] = m.patches[p].p.kind;
        const std::vector<pgd::Tables32> tv(1, t);
        const picgpu_status us = upload(c, &c->t32, tv);
        if (us) return us;
    }
    if (c->mixed) {
        // in-cell mover: dt per cell size along each axis (uniform block
        // meshes: class 0's corner 6 sits at +h/2)
        for (int a = 0; a < 3; ++a) {
            const double h = 2.0 * m.cls_offset[3 * 6 + a];
            c->cell_keep[a] = m.empty[a] ? 0.f : 1.f;
            c->cell_dth[a] = m.empty[a] ? 0.f : float(cfg->dt / h);
        }
        picgpu_status us;
        c->xq_cap = 16 * c->sm_count;
        if ((us = dalloc(c, &c->xq_count, size_t(c->xq_cap))) || (us = dalloc(c, &c->xq_start, size_t(c->xq_cap))))
            return us;
    }
    CK(pgd::fields_set_patches(c->pc));
    CK(pgd::collide_set_tables(c->tc));

    // mesh arrays
    picgpu_status s;
    DMesh& d = c->dm;
    d.n_cells = m.n_cells;
    d.n_points = m.n_points;
    d.n_bfaces = int(m.bfaces.size());
    d.n_classes = m.n_classes;
    for (int a = 0; a < 3; ++a) {
        d.empty[a] = m.empty[a];
        d.mesh_centre[a] = m.mesh_centre[a];
    }
    d.any_empty = m.empty[0] || m.empty[1] || m.empty[2];
    std::vector<float> inv32(m.cls_tetinv.begin(), m.cls_tetinv.end());
    std::vector<float> off32(m.cls_offset.begin(), m.cls_offset.end());
    std::vector<float> fn32(m.cls_fnormal.begin(), m.cls_fnormal.end());
    std::vector<int> bf_cell, bf_patch;
    std::vector<double> bf_normal, bf_area, bf_delta;
    for (const auto& bf : m.bfaces) {
        bf_cell.push_back(bf.cell);
        bf_patch.push_back(bf.patch);
        for (int a = 0; a < 3; ++a) bf_normal.push_back(bf.normal[a]);
        bf_area.push_back(bf.area);
        bf_delta.push_back(bf.delta);
    }
    std::vector<double> Mdiag(m.n_cells), Moff(m.lap_off.size()), dinv(m.n_cells);
    for (int i = 0; i < m.n_cells; ++i) Mdiag[i] = -m.lap_diag[i];
    pg::circuit_add_diagonal(m, cfg->circuit, cfg->dt, Mdiag);
    for (int i = 0; i < m.n_cells; ++i) dinv[i] = 1.0 / Mdiag[i];
    for (size_t i = 0; i < Moff.size(); ++i) Moff[i] = -m.lap_off[i];
    int* ip;
    double* dp;
    float* fp;
#define UP(field, vec, T)                              \
    {                                                  \
        T* ptr_;                                       \
        if ((s = upload(c, &ptr_, vec))) return s;     \
        d.field = ptr_;                                \
    }
    UP(cell_class, m.cell_class, int);
    UP(nbr, m.nbr, int);
    UP(cell_pt, m.cell_pt, int);
    UP(cc, m.cc, double);
    std::vector<float> cc32(m.cc.begin(), m.cc.end());
    UP(cc32, cc32, float);
    UP(vol, m.vol, double);
    UP(tetinv, m.cls_tetinv, double);
    UP(tetinv32, inv32, float);
    UP(offset, m.cls_offset, double);
    UP(offset32, off32, float);
    UP(fnormal, m.cls_fnormal, double);
    UP(fnormal32, fn32, float);
    UP(farea, m.cls_farea, double);
    UP(ip_weight, m.ip_weight, double);
    UP(cell_bface, m.cell_bface, int);
    UP(bf_cell, bf_cell, int);
    UP(bf_patch, bf_patch, int);
    UP(bf_normal, bf_normal, double);
    UP(bf_area, bf_area, double);
    UP(bf_delta, bf_delta, double);
    UP(vw_weight, m.vw_weight, double);
    UP(pi_start, m.pi_start, int);
    UP(pi_src, m.pi_src, int);
    UP(pi_w, m.pi_w, double);
    UP(Mdiag, Mdiag, double);
    UP(Moff, Moff, double);
    UP(dinv, dinv, double);
    UP(pc_start, m.pc_start, int);
    UP(pc_slot, m.pc_slot, int);
    d.uniform = m.n_classes == 1;
    // one M coefficient per face direction: the SpMV then skips Moff
    d.lap_uniform = 1;
    for (int f = 0; f < 6; ++f) d.lap_coef[f] = 0.0;
    {
        bool seen[6] = {};
        for (size_t k = 0; k < Moff.size() && d.lap_uniform; ++k) {
            if (m.nbr[k] < 0) continue;
            const int f = int(k % 6);
            if (!seen[f]) { seen[f] = true; d.lap_coef[f] = Moff[k]; }
            else if (Moff[k] != d.lap_coef[f]) d.lap_uniform = 0;
        }
    }
#undef UP
    (void)ip; (void)dp; (void)fp;

    // fields
    const size_t nc = m.n_cells, np = m.n_points, nbf = m.bfaces.size(), npa = m.patches.size();
    if ((s = dalloc(c, &c->phi, nc)) || (s = dalloc(c, &c->rho, nc)) || (s = dalloc(c, &c->E, 3 * nc)) ||
        (s = dalloc(c, &c->Ept, 3 * np)) || (s = dalloc(c, &c->Eb, 3 * nbf)) ||
        (s = dalloc(c, &c->E32, 3 * nc)) || (s = dalloc(c, &c->Ept32, 3 * np)) ||
        (s = dalloc(c, &c->cc_data, nc)) || (s = dalloc(c, &c->vtx_data, np)) ||
        (s = dalloc(c, &c->cc_fix, nc)) || (s = dalloc(c, &c->vtx_fix, np)) ||
        (s = dalloc(c, &c->qconv, npa)) || (s = dalloc(c, &c->sigma, npa)) ||
        (s = dalloc(c, &c->grad_bc, npa)) || (s = dalloc(c, &c->b, nc)) || (s = dalloc(c, &c->r, nc)) ||
        (s = dalloc(c, &c->z, nc)) || (s = dalloc(c, &c->p[0], nc)) || (s = dalloc(c, &c->p[1], nc)) ||
        (s = dalloc(c, &c->q, nc)) || (s = dalloc(c, &c->part, 4 * size_t(pgd::pcg_blocks(int(nc))) + 8)) ||
        (s = dalloc(c, &c->st, 1)) || (s = dalloc(c, &c->counters, PICGPU_MAX_SPECIES)) ||
        (s = dalloc(c, &c->diag, 64)) || (s = dalloc(c, &c->n_dev, PICGPU_MAX_SPECIES)) ||
        (s = dalloc(c, &c->first_dev, PICGPU_MAX_SPECIES)) || (s = dalloc(c, &c->step_dev, 1)) ||
        (s = dalloc(c, &c->inj_flag, 1)))
        return s;
    if (c->mixed && ((s = dalloc(c, &c->acc9, size_t(cfg->n_species) * 9 * nc)) ||
                     (s = dalloc(c, &c->Ec4, 9 * nc))))
        return s;
    if (c->Ec4) CK(cudaMemset(c->Ec4, 0, 9 * nc * sizeof(float4)));
    CK(cudaMemset(c->phi, 0, nc * sizeof(double)));
    CK(cudaMemset(c->E, 0, 3 * nc * sizeof(double)));
    CK(cudaMemset(c->Ept, 0, 3 * np * sizeof(double)));
    CK(cudaMemset(c->E32, 0, 3 * nc * sizeof(float)));
    CK(cudaMemset(c->Ept32, 0, 3 * np * sizeof(float)));
    CK(cudaMemset(c->qconv, 0, npa * sizeof(double)));
    CK(cudaMemset(c->sigma, 0, npa * sizeof(double)));
    CK(cudaMemset(c->grad_bc, 0, npa * sizeof(double)));
    if (cfg->circuit.model != PICGPU_CIRCUIT_NONE) {
        const pg::CircuitState st0 = pg::circuit_start(cfg->circuit);
        std::vector<int> faces = pg::circuit_cathode_faces(m, cfg->circuit);
        int* fd = nullptr;
        if ((s = upload(c, &fd, faces)) || (s = dalloc(c, &c->circ_state, 1))) return s;
        c->circ.faces = fd;
        c->circ.n_faces = int(faces.size());
        CK(cudaMemcpy(c->circ_state, &st0, sizeof st0, cudaMemcpyHostToDevice));
        if (cfg->circuit.model == PICGPU_CIRCUIT_IDEAL_CURRENT) {
            // circuitBoundary's stored gradient: sigma / epsilon0
            const double g0 = st0.sigma / (1.0 / (kMu0 * kCl * kCl));
            CK(cudaMemcpy(c->grad_bc + cfg->circuit.cathode_patch, &g0, sizeof g0, cudaMemcpyHostToDevice));
        }
    }
    CK(cudaMemset(c->st, 0, sizeof(pgd::PcgState)));
    CK(cudaMallocHost(&c->st_host, sizeof(pgd::PcgState)));
    CK(cudaMallocHost(&c->counters_host, sizeof(pgd::MoveCounters) * PICGPU_MAX_SPECIES));
    std::memset(c->st_host, 0, sizeof(pgd::PcgState));
    std::memset(c->counters_host, 0, sizeof(pgd::MoveCounters) * PICGPU_MAX_SPECIES);
    long max_hint = 0;
    for (int sp = 0; sp < cfg->n_species; ++sp) {
        const long cap = std::max<long>(cfg->species[sp].capacity_hint, 1024);
        if ((s = alloc_species(c, sp, cap))) return s;
        max_hint = std::max<long>(max_hint, cfg->species[sp].capacity_hint);
    }
    // with a capacity hint, the staging of host arrays is sized here too, so
    // that the first picgpu_set_particles allocates nothing
    if (max_hint > 0 && (s = ensure_rows(c, size_t(max_hint)))) return s;
    if (cfg->maxwell_solver != PICGPU_MAXWELL_ELECTROSTATIC)
        if ((s = set_applied_field(c))) return s;
    std::string msg;
    const int cs = pgd::collide_init(c->coll, c->cfg, c->dm, c->stream, &msg);
    if (cs) return bad(c, picgpu_status(cs), msg);
    if (cfg->perez.enabled) {
        // ionisation raises an ion's charge modifier and adds electrons with
        // the ion's nParticle (PerezIonizationModel.C:336-346)
        if (c->n_cases > 1) return bad(c, PICGPU_NOT_SUPPORTED, "Perez ionisation is not supported with ensembles");
        if ((s = enable_attributes(c, cfg->electron_species))) return s;
        for (int k = 0; k < cfg->perez.n_ions; ++k)
            if ((s = enable_attributes(c, cfg->perez.ion[k].species))) return s;
    }
    if (cfg->merging.enabled) {
        // merged parcels carry their summed nParticle (PairMerging.C:210-214)
        if (c->n_cases > 1) return bad(c, PICGPU_NOT_SUPPORTED, "PairMerging is not supported with ensembles");
        for (int k = 0; k < cfg->merging.n_species; ++k)
            if ((s = enable_attributes(c, cfg->merging.species[k]))) return s;
    }
    if (cfg->learned.enabled) {
        if (cfg->maxwell_solver != PICGPU_MAXWELL_ELECTROSTATIC)
            return bad(c, PICGPU_INVALID_ARG, "learned warm start needs the electrostatic Maxwell solver");
        c->ws = std::make_unique<pgd::LearnedWarmStart>();
        const int ls = c->ws->init(cfg->learned, cfg->seed, c->m.n_cells, c->m.n, c->m.cell_ijk, c->stream, &msg);
        if (ls) return bad(c, picgpu_status(ls), msg);
    }
    if (cfg->pcg_precond == PICGPU_PRECOND_MULTIGRID && cfg->maxwell_solver == PICGPU_MAXWELL_ELECTROSTATIC) {
        pgd::MgSettings ms;
        if (cfg->mg.pre_sweeps > 0) ms.pre = cfg->mg.pre_sweeps;
        if (cfg->mg.post_sweeps > 0) ms.post = cfg->mg.post_sweeps;
        if (cfg->mg.coarsest_cells > 0) ms.coarsest = cfg->mg.coarsest_cells;
        if (cfg->mg.omega > 0) ms.omega = cfg->mg.omega;
        if (cfg->mg.scale_correction > 0) ms.scale = cfg->mg.scale_correction;
        if (ms.pre > 8 || ms.post > 8 || ms.coarsest > 4096 || !(ms.omega < 2.0) || !(ms.scale <= 2.0))
            return bad(c, PICGPU_INVALID_ARG, "config: multigrid settings out of range");
        std::vector<double> Md(c->m.n_cells), Mo(c->m.lap_off.size());
        for (int i = 0; i < c->m.n_cells; ++i) Md[i] = -c->m.lap_diag[i];
        pg::circuit_add_diagonal(c->m, cfg->circuit, cfg->dt, Md);
        for (size_t i = 0; i < Mo.size(); ++i) Mo[i] = -c->m.lap_off[i];
        c->mg = std::make_unique<pgd::MultigridPCG>();
        if (!c->mg->init(c->m, Md, Mo, ms, &msg)) return bad(c, PICGPU_NOT_SUPPORTED, msg);
    }
    c->stager.init();  // pinned ring for caller arrays (on failure, plain copies)
    CK(cudaStreamSynchronize(c->stream));
    c->err.clear();
    return PICGPU_OK;
}

void picgpu_destroy(picgpu_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->mg.reset();
    pgd::collide_free(c->coll);
    for (void* a : c->allocs)
        if (a) cudaFree(a);
    for (auto& ep : c->pending) { cudaEventDestroy(ep.a); cudaEventDestroy(ep.b); }
    for (auto e : c->free_events) cudaEventDestroy(e);
    if (c->timer[0]) { cudaEventDestroy(c->timer[0]); cudaEventDestroy(c->timer[1]); }
    if (c->pcg_graph) cudaGraphExecDestroy(c->pcg_graph);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    if (c->replay_ev[0]) { cudaEventDestroy(c->replay_ev[0]); cudaEventDestroy(c->replay_ev[1]); }
    if (c->st_host) cudaFreeHost(c->st_host);
    if (c->counters_host) cudaFreeHost(c->counters_host);
    c->stager.release();
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* picgpu_last_error(const picgpu_ctx* c) { return c ? c->err.c_str() : "null context"; }

picgpu_status picgpu_mesh_query(const picgpu_ctx* c, picgpu_mesh_info* info) {
    if (!c || !info) return PICGPU_INVALID_ARG;
    info->n_cells = c->m.n_cells;
    info->n_points = c->m.n_points;
    info->n_tets = 12LL * c->m.n_cells;
    info->n_patches = (int64_t)c->m.patches.size();
    return PICGPU_OK;
}


picgpu_status picgpu_set_particles(picgpu_ctx* c, int species, size_t n, const int32_t* tet,
                                   const double* bary, const double* U) {
    if (!c || species < 0 || species >= c->cfg.n_species) return PICGPU_INVALID_ARG;
    if (n && (!tet || !bary || !U)) return PICGPU_INVALID_ARG;
    if (n > size_t(1) << 31) return bad(c, PICGPU_INVALID_ARG, "at most 2^31 particles per species");
    picgpu_status s;
    if ((s = ensure_rows(c, n))) return s;
    // the rows go to the device as they are; the checks and the column
    // conversion run there
    if (n) {
        CK(c->stager.upload(c->rows_tet, tet, n * sizeof(int32_t), c->stream));
        CK(c->stager.upload(c->rows_y, bary, 3 * n * sizeof(double), c->stream));
        CK(c->stager.upload(c->rows_u, U, 3 * n * sizeof(double), c->stream));
        CK(cudaMemsetAsync(c->inj_flag, 0, sizeof(int), c->stream));
        pgd::launch_check_tets(c->rows_tet, long(n), 12LL * c->m.n_cells, c->inj_flag, c->stream);
        int badt = 0;
        CK(cudaMemcpyAsync(&badt, c->inj_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (badt) return bad(c, PICGPU_INVALID_ARG, "particles: tet index out of range");
    }
    SpeciesBuf& B = c->sp[species];
    if (long(n) > B.cap) {
        const long cap = std::max<long>(long(n) + long(n) / 4, c->cfg.species[species].capacity_hint);
        if ((s = alloc_species(c, species, cap))) return s;
    }
    B.cur = 0;
    B.n = long(n);
    B.alive = long(n);
    pgd::launch_scatter_rows(c->rows_tet, c->rows_y, c->rows_u, long(n), view(c, species, 0), c->mixed, c->stream);
    // new parcels: the species weight and charge modifier 1
    pgd::launch_fill_attributes(view(c, species, 0), 0, long(n), c->cfg.species[species].weight, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return PICGPU_OK;
}

picgpu_status picgpu_count_particles(picgpu_ctx* c, int species, size_t* n) {
    if (!c || !n || species < 0 || species >= c->cfg.n_species) return PICGPU_INVALID_ARG;
    *n = size_t(c->sp[species].alive);
    return PICGPU_OK;
}

picgpu_status picgpu_get_particles(picgpu_ctx* c, int species, size_t cap, int32_t* tet, double* bary,
                                   double* U, size_t* nout) {
    if (!c || !nout || species < 0 || species >= c->cfg.n_species) return PICGPU_INVALID_ARG;
    CK(cudaStreamSynchronize(c->stream));
    SpeciesBuf& B = c->sp[species];
    // compact into the scratch half of the double buffer (the store itself is
    // left as it is), then rows on the device, one copy per array
    pgd::DSpecies src = view(c, species, B.cur);
    long kept = B.n;
    if (B.n > 0) {
        const long nblk = pgd::compact_blocks(B.n);
        picgpu_status st = ensure_scan(c, nblk + 1);
        if (st) return st;
        const pgd::DSpecies dst = view(c, species, B.cur ^ 1);
        CK(pgd::compact_species(src, dst, B.n, c->mixed, c->scan_buf, &kept, c->stream));
        c->launches += 3;
        src = dst;
    }
    *nout = size_t(kept);
    if (!tet) return PICGPU_OK;
    if (cap < size_t(kept) || !bary || !U) return PICGPU_INVALID_ARG;
    picgpu_status st = ensure_rows(c, size_t(kept));
    if (st) return st;
    pgd::launch_gather_rows(src, kept, c->mixed, c->rows_tet, c->rows_y, c->rows_u, c->stream);
    if (kept) {
        CK(c->stager.download(tet, c->rows_tet, size_t(kept) * sizeof(int32_t), c->stream));
        CK(c->stager.download(bary, c->rows_y, 3 * size_t(kept) * sizeof(double), c->stream));
        CK(c->stager.download(U, c->rows_u, 3 * size_t(kept) * sizeof(double), c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_set_parcel_attributes(picgpu_ctx* c, int species, size_t n, const double* nParticle,
                                           const int32_t* chargeModifier) {
    if (!c || species < 0 || species >= c->cfg.n_species) return PICGPU_INVALID_ARG;
    if (n && (!nParticle || !chargeModifier)) return PICGPU_INVALID_ARG;
    SpeciesBuf& B = c->sp[species];
    const double w = c->cfg.species[species].weight;
    for (size_t i = 0; i < n; ++i) {
        // a parcel's weight multiple of the species weight and its charge
        // modifier scale the fixed-point charge deposit: both are bounded
        if (!(nParticle[i] > 0.0) || !(nParticle[i] <= 4096.0 * w) || chargeModifier[i] < 0 ||
            chargeModifier[i] > 1024)
            return bad(c, PICGPU_INVALID_ARG,
                       "parcel attributes: nParticle in (0, 4096 w] and chargeModifier in [0, 1024]");
    }
    CK(cudaStreamSynchronize(c->stream));
    // the attributes follow the order of picgpu_get_particles: the store is
    // compacted first
    picgpu_status st;
    if ((st = compact(c, true))) return st;
    if (size_t(B.n) != n) return bad(c, PICGPU_INVALID_ARG, "parcel attributes: n differs from the parcel count");
    if ((st = enable_attributes(c, species))) return st;
    if (n) {
        CK(cudaMemcpyAsync(B.nw[B.cur], nParticle, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(B.zq[B.cur], chargeModifier, n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_get_parcel_attributes(picgpu_ctx* c, int species, size_t cap, double* nParticle,
                                           int32_t* chargeModifier, size_t* nout) {
    if (!c || !nout || species < 0 || species >= c->cfg.n_species) return PICGPU_INVALID_ARG;
    CK(cudaStreamSynchronize(c->stream));
    SpeciesBuf& B = c->sp[species];
    picgpu_status st;
    if ((st = compact(c, true))) return st;
    *nout = size_t(B.n);
    if (!nParticle) return PICGPU_OK;
    if (cap < size_t(B.n) || !chargeModifier) return PICGPU_INVALID_ARG;
    if (!B.attrs) {
        for (long i = 0; i < B.n; ++i) {
            nParticle[i] = c->cfg.species[species].weight;
            chargeModifier[i] = 1;
        }
        return PICGPU_OK;
    }
    if (B.n) {
        CK(cudaMemcpyAsync(nParticle, B.nw[B.cur], size_t(B.n) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(chargeModifier, B.zq[B.cur], size_t(B.n) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_set_step_index(picgpu_ctx* c, int64_t steps_done) {
    if (!c || steps_done < 0) return PICGPU_INVALID_ARG;
    c->step_index = steps_done;
    return PICGPU_OK;
}

picgpu_status picgpu_compute_field(picgpu_ctx* c) {
    if (!c) return PICGPU_INVALID_ARG;
    picgpu_status s;
    if (c->cfg.maxwell_solver != PICGPU_MAXWELL_ELECTROSTATIC) return PICGPU_OK;
    if ((s = efield(c))) return s;
    CK(cudaStreamSynchronize(c->stream));
    if (c->profiling) harvest_events(c);
    return PICGPU_OK;
}

picgpu_status picgpu_initialise_fields(picgpu_ctx* c) {
    if (!c) return PICGPU_INVALID_ARG;
    picgpu_status s;
    if ((s = zero_accumulators(c))) return s;
    if ((s = move_species(c, true))) return s;
    if ((s = charge_update(c))) return s;
    if ((s = solve_fields(c, nullptr))) return s;
    CK(cudaStreamSynchronize(c->stream));
    if (c->profiling) harvest_events(c);
    return PICGPU_OK;
}

// ------------------------------------------------------- injection ------
picgpu_status picgpu_set_injection(picgpu_ctx* c, int n, const picgpu_injection* inj) {
    if (!c || n < 0 || n > PICGPU_MAX_INJECTORS || (n > 0 && !inj)) return PICGPU_INVALID_ARG;
    if (c->n_cases != 1) return bad(c, PICGPU_NOT_SUPPORTED, "injection: not for ensemble contexts");
    for (Injector& I : c->injectors) {
        dfree(c, I.tri_cum);
        dfree(c, I.tri_cell);
        dfree(c, I.tri_tet);
        dfree(c, I.tri_normal);
        dfree(c, I.tri_fc);
    }
    c->injectors.clear();
    for (int i = 0; i < n; ++i) {
        const picgpu_injection& q = inj[i];
        if (q.patch < 0 || q.patch >= int(c->m.patches.size()))
            return bad(c, PICGPU_INVALID_ARG, "injection: no such patch");
        const int kind = c->m.patches[q.patch].p.kind;
        if (kind == PICGPU_PATCH_CYCLIC || kind == PICGPU_PATCH_EMPTY)
            return bad(c, PICGPU_INVALID_ARG, "injection: the patch must not be cyclic or empty");
        if (q.velocity_model < PICGPU_EMIT_BIRD_MAXWELLIAN_FLUX || q.velocity_model > PICGPU_EMIT_HALF_MAXWELLIAN_FLUX)
            return bad(c, PICGPU_INVALID_ARG, "injection: unknown velocityModel");
        if (q.n_species < 0 || q.n_species > PICGPU_MAX_SPECIES)
            return bad(c, PICGPU_INVALID_ARG, "injection: injectionTypeIds");
        for (int j = 0; j < q.n_species; ++j) {
            if (q.species[j] < 0 || q.species[j] >= c->cfg.n_species || !(c->cfg.species[q.species[j]].weight > 0))
                return bad(c, PICGPU_INVALID_ARG, "injection: species not defined");
            if (!(q.frequency[j] >= 0) || !(q.eV[j] >= 0))
                return bad(c, PICGPU_INVALID_ARG, "injection: frequencies and eV must be >= 0");
        }
        const pg::PatchTriangles T = pg::patch_triangles(c->m, q.patch);
        if (T.cell.empty()) return bad(c, PICGPU_INVALID_ARG, "injection: the patch has no boundary faces");
        Injector I;
        I.cfg = q;
        I.n_tri = int(T.cell.size());
        I.area = T.area;
        picgpu_status st;
        c->injectors.push_back(I);
        Injector& J = c->injectors.back();
        if ((st = upload(c, &J.tri_cum, T.cum)) || (st = upload(c, &J.tri_cell, T.cell)) ||
            (st = upload(c, &J.tri_tet, T.tet)) || (st = upload(c, &J.tri_normal, T.normal)) ||
            (st = upload(c, &J.tri_fc, T.centre)))
            return st;
    }
    if (!c->inj_err) {
        picgpu_status st = dalloc(c, &c->inj_err, 1);
        if (st) return st;
    }
    CK(cudaMemset(c->inj_err, 0, sizeof(int)));
    return PICGPU_OK;
}

picgpu_status picgpu_set_freestream(picgpu_ctx* c, int n, const picgpu_freestream* fs) {
    if (!c || n < 0 || n > PICGPU_MAX_FREESTREAMS || (n > 0 && !fs)) return PICGPU_INVALID_ARG;
    if (c->n_cases != 1) return bad(c, PICGPU_NOT_SUPPORTED, "freestream: not for ensemble contexts");
    for (int i = 0; i < n; ++i) {
        const std::string e = pg::check_freestream(c->m, c->cfg, fs[i]);
        if (!e.empty()) return bad(c, PICGPU_INVALID_ARG, e);
        for (int j = 0; j < fs[i].n_species; ++j)
            if (!(c->cfg.species[fs[i].species[j]].weight > 0))
                return bad(c, PICGPU_INVALID_ARG, "freestream: species without a weight");
    }
    for (FsInjector& Z : c->freestreams) {
        for (void* p : {(void*)Z.cell, (void*)Z.tet0, (void*)Z.frac0, (void*)Z.n_in, (void*)Z.t1, (void*)Z.t2,
                        (void*)Z.add, (void*)Z.s, (void*)Z.acc, (void*)Z.counts, (void*)Z.offsets, (void*)Z.sums})
            dfree(c, p);
    }
    c->freestreams.clear();
    for (int i = 0; i < n; ++i) {
        c->freestreams.emplace_back();
        FsInjector& Z = c->freestreams.back();
        Z.cfg = fs[i];
        Z.F = pg::freestream_faces(c->m, c->cfg, fs[i]);
        const size_t nf = size_t(Z.F.n_faces);
        picgpu_status st;
        if ((st = upload(c, &Z.cell, Z.F.cell)) || (st = upload(c, &Z.tet0, Z.F.tet0)) ||
            (st = upload(c, &Z.frac0, Z.F.frac0)) || (st = upload(c, &Z.n_in, Z.F.n_in)) ||
            (st = upload(c, &Z.t1, Z.F.t1)) || (st = upload(c, &Z.t2, Z.F.t2)) || (st = upload(c, &Z.add, Z.F.add)) ||
            (st = upload(c, &Z.s, Z.F.s)) || (st = dalloc(c, &Z.acc, nf * Z.F.n_species)) ||
            (st = dalloc(c, &Z.counts, nf)) || (st = dalloc(c, &Z.offsets, nf + 1)) ||
            (st = dalloc(c, &Z.sums, size_t(pgd::init_scan_scratch(int(nf))) + 1)))
            return st;
        CK(cudaMemset(Z.acc, 0, nf * Z.F.n_species * sizeof(double)));
    }
    if (!c->inj_err) {
        picgpu_status st = dalloc(c, &c->inj_err, 1);
        if (st) return st;
    }
    CK(cudaMemset(c->inj_err, 0, sizeof(int)));
    return PICGPU_OK;
}

picgpu_status picgpu_set_emission(picgpu_ctx* c, int n, const picgpu_emission* em) {
    if (!c || n < 0 || n > PICGPU_MAX_EMISSIONS || (n > 0 && !em)) return PICGPU_INVALID_ARG;
    if (c->n_cases != 1) return bad(c, PICGPU_NOT_SUPPORTED, "emission: not for ensemble contexts");
    const int es = c->cfg.electron_species;
    for (int i = 0; i < n; ++i) {
        const picgpu_emission& q = em[i];
        if (es < 0 || es >= c->cfg.n_species || c->cfg.species[es].charge == 0.0)
            return bad(c, PICGPU_INVALID_ARG, "emission: the config names no charged electron species");
        if (q.patch < 0 || q.patch >= int(c->m.patches.size()))
            return bad(c, PICGPU_INVALID_ARG, "emission: no such patch");
        const int kind = c->m.patches[q.patch].p.kind;
        if (kind == PICGPU_PATCH_CYCLIC || kind == PICGPU_PATCH_EMPTY)
            return bad(c, PICGPU_INVALID_ARG, "emission: the patch must not be cyclic or empty");
        if (q.model != PICGPU_EMISSION_THERMIONIC && q.model != PICGPU_EMISSION_FOWLER_NORDHEIM)
            return bad(c, PICGPU_INVALID_ARG, "emission: unknown model");
        if (!(q.work_function > 0.0)) return bad(c, PICGPU_INVALID_ARG, "emission: fnW must be > 0");
        if (q.model == PICGPU_EMISSION_THERMIONIC && !(q.temperature > 0.0 && q.lambda_r >= 0.0))
            return bad(c, PICGPU_INVALID_ARG, "emission: thermionic emission needs T > 0 and lambdaR >= 0");
        if (q.weight > 0.0 && q.weight != c->cfg.species[es].weight)
            return bad(c, PICGPU_INVALID_ARG,
                       "emission: nParticle must equal the electron species' weight (one weight per species)");
    }
    for (Injector& I : c->emitters) {
        for (void* p : {(void*)I.tri_cum, (void*)I.tri_cell, (void*)I.tri_tet, (void*)I.tri_normal,
                        (void*)I.tri_fc, (void*)I.em_faces})
            dfree(c, p);
    }
    c->emitters.clear();
    for (int i = 0; i < n; ++i) {
        const picgpu_emission& q = em[i];
        const pg::PatchTriangles T = pg::patch_triangles(c->m, q.patch);
        if (T.cell.empty()) return bad(c, PICGPU_INVALID_ARG, "emission: the patch has no boundary faces");
        c->emitters.emplace_back();
        Injector& J = c->emitters.back();
        J.em = q;
        J.n_tri = int(T.cell.size());
        J.area = T.area;
        if (q.model == PICGPU_EMISSION_THERMIONIC)
            J.em_j = pg::thermionic_current(q.lambda_r, q.temperature, q.work_function,
                                            std::fabs(c->cfg.species[es].charge));
        std::vector<int> faces;
        for (size_t b = 0; b < c->m.bfaces.size(); ++b)
            if (c->m.bfaces[b].patch == q.patch) faces.push_back(int(b));
        J.em_n_faces = int(faces.size());
        picgpu_status st;
        if ((st = upload(c, &J.tri_cum, T.cum)) || (st = upload(c, &J.tri_cell, T.cell)) ||
            (st = upload(c, &J.tri_tet, T.tet)) || (st = upload(c, &J.tri_normal, T.normal)) ||
            (st = upload(c, &J.tri_fc, T.centre)) || (st = upload(c, &J.em_faces, faces)))
            return st;
    }
    picgpu_status st;
    if (!c->em_sum && (st = dalloc(c, &c->em_sum, 1))) return st;
    if (!c->inj_err) {
        if ((st = dalloc(c, &c->inj_err, 1))) return st;
    }
    CK(cudaMemset(c->inj_err, 0, sizeof(int)));
    return PICGPU_OK;
}

// ------------------------------------------------ initial conditions ----
// picInitialise (preProcess/picInitialise/picInitialise.C:30-319) for a
// context; the placement runs on the device (csrc/init.cu).
namespace {

constexpr double kBoltzmann = 1.380649e-23;
constexpr double kElementary = 1.602176634e-19;

}  // namespace

picgpu_status picgpu_initialise(picgpu_ctx* c, const picgpu_init* in, picgpu_init_stats* st) {
    if (!c || !in) return PICGPU_INVALID_ARG;
    const int ns = c->cfg.n_species;
    if (in->model < PICGPU_INIT_NONE || in->model > PICGPU_INIT_UNIFORM_DISPLACEMENT)
        return bad(c, PICGPU_INVALID_ARG, "initialise: unknown InitializationModel");
    if (c->n_cases != 1) return bad(c, PICGPU_NOT_SUPPORTED, "initialise: not for ensemble contexts");
    picgpu_init_stats S{};
    picgpu_status ps;
    const pg::HexMesh& m = c->m;
    if (in->clear_particles)
        for (int sp = 0; sp < ns; ++sp) {
            c->sp[sp].n = 0;
            c->sp[sp].alive = 0;
            c->sp[sp].cur = 0;
        }

    // per-species sampling (what each model draws)
    pgd::InitSpecies smp[PICGPU_MAX_SPECIES] = {};
    bool place[PICGPU_MAX_SPECIES] = {};
    bool calc_T = false, calc_n = false;
    for (int sp = 0; sp < ns; ++sp) {
        const picgpu_species& P = c->cfg.species[sp];
        pgd::InitSpecies& q = smp[sp];
        q.n = in->number_density[sp];
        q.w = P.weight;
        const double th = std::sqrt(kBoltzmann * in->temperature[sp] / P.mass);  // equipartitionLinearVelocity
        switch (in->model) {
            case PICGPU_INIT_EQUIPARTITION:
                for (int a = 0; a < 3; ++a) { q.scale[a] = th; q.drift[a] = in->velocity[a]; }
                place[sp] = q.n > 0;
                break;
            case PICGPU_INIT_MAXWELLIAN:
                for (int a = 0; a < 3; ++a) { q.scale[a] = in->thermal_velocity[sp][a]; q.drift[a] = in->drift_velocity[sp][a]; }
                place[sp] = q.n > 0;
                calc_T = true;
                break;
            case PICGPU_INIT_ISOTROPIZATION: {
                const double f = in->tperp_over_tpara;
                if (!(f > 0)) return bad(c, PICGPU_INVALID_ARG, "initialise: Tperp_over_Tpara must be > 0");
                const double T = in->temperature[sp];
                const double upara = std::sqrt(kBoltzmann * T / (((2.0 / 3.0) * f + (1.0 / 3.0)) * P.mass));
                const double uperp = std::sqrt(kBoltzmann * T / (((2.0 / 3.0) + (1.0 / (3.0 * f))) * P.mass));
                q.scale[0] = upara;
                q.scale[1] = uperp;
                q.scale[2] = uperp;
                place[sp] = q.n > 0;
                break;
            }
            case PICGPU_INIT_QUASINEUTRAL_PLASMA:
                for (int a = 0; a < 3; ++a) q.scale[a] = th;
                q.speed = std::sqrt(in->temperature[sp] * kBoltzmann * 3.0 / P.mass);
                calc_n = true;
                break;
            case PICGPU_INIT_UNIFORM_DISPLACEMENT:
                for (int a = 0; a < 3; ++a) q.scale[a] = th;
                q.displacement = in->displacement[sp];
                place[sp] = (in->species_mask >> sp) & 1;
                calc_n = true;
                break;
            default:
                calc_T = calc_n = true;
                break;
        }
        if (place[sp] && !(P.weight > 0)) return bad(c, PICGPU_INVALID_ARG, "initialise: species weight must be > 0");
    }
    if (in->model == PICGPU_INIT_QUASINEUTRAL_PLASMA) {
        const int ion = in->ion_species, el = c->cfg.electron_species;
        if (ion < 0 || ion >= ns) return bad(c, PICGPU_INVALID_ARG, "initialise: ionSpecies is not defined");
        if (el < 0 || el >= ns) return bad(c, PICGPU_INVALID_ARG, "initialise: electron species is not defined");
        if (c->cfg.species[ion].charge + c->cfg.species[el].charge != 0.0)
            return bad(c, PICGPU_INVALID_ARG,
                       "initialise: ion and electron charge must be of same magnitude and opposite signs");
        for (int sp : {ion, el}) {
            const double nn = in->cell_count / c->cfg.species[sp].weight;
            if (!(nn >= 0 && nn < 2147483647.0)) return bad(c, PICGPU_CAPACITY, "initialise: cellCount too large");
            smp[sp].cell_count = int(nn);
            place[sp] = smp[sp].cell_count > 0;
        }
    }

    // lattice of UniformDisplacement (UniformInitialization.C:60-87)
    double lo[3], hi[3], glo[3], ghi[3], dir[3], delta[3], span_len = 0;
    const int gtop = pg::grid_point_id(m, m.n[0], m.n[1], m.n[2]);
    for (int a = 0; a < 3; ++a) {
        glo[a] = m.grid_pts[a];
        ghi[a] = m.grid_pts[3 * size_t(gtop) + a];
        lo[a] = in->use_bounds ? in->min[a] : glo[a];
        hi[a] = in->use_bounds ? in->max[a] : ghi[a];
    }
    if (in->model == PICGPU_INIT_UNIFORM_DISPLACEMENT) {
        const double dm = std::sqrt(in->displacement_dir[0] * in->displacement_dir[0] +
                                    in->displacement_dir[1] * in->displacement_dir[1] +
                                    in->displacement_dir[2] * in->displacement_dir[2]);
        if (!(dm > 0)) return bad(c, PICGPU_INVALID_ARG, "initialise: displacementDir must be non-zero");
        for (int a = 0; a < 3; ++a) dir[a] = in->displacement_dir[a] / dm;
        double span[3];
        for (int a = 0; a < 3; ++a) span[a] = hi[a] - lo[a];
        span_len = span[0] * dir[0] + span[1] * dir[1] + span[2] * dir[2];
        for (int a = 0; a < 3; ++a) {
            if (in->particle_numbers[a] < 0) return bad(c, PICGPU_INVALID_ARG, "initialise: particleNumbers < 0");
            delta[a] = span[a] / double(std::max<long long>(in->particle_numbers[a] - 1, 2));
        }
    }

    int* counts = nullptr;
    long long *offsets = nullptr, *sums = nullptr, *mm = nullptr;
    int* err = nullptr;
    const int nc = m.n_cells;
    auto release = [&]() {
        dfree(c, counts);
        dfree(c, offsets);
        dfree(c, sums);
        dfree(c, mm);
        dfree(c, err);
    };
    if ((ps = dalloc(c, &counts, size_t(nc))) || (ps = dalloc(c, &offsets, size_t(nc) + 1)) ||
        (ps = dalloc(c, &sums, size_t(pgd::init_scan_scratch(nc)) + 1)) || (ps = dalloc(c, &mm, 3)) ||
        (ps = dalloc(c, &err, 1))) {
        release();
        return ps;
    }
    CK(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float place_ms = 0;
    const bool constrain = m.empty[0] || m.empty[1] || m.empty[2];
    for (int sp = 0; sp < ns && in->model != PICGPU_INIT_NONE; ++sp) {
        if (!place[sp]) continue;
        pgd::InitParams P{};
        P.m = c->dm;
        P.model = in->model;
        P.species = sp;
        P.constrain = constrain && in->model != PICGPU_INIT_UNIFORM_DISPLACEMENT;
        P.use_maxwellian = in->use_maxwellian;
        P.seed = in->seed;
        P.sp = smp[sp];
        P.tet_vol = c->tet_vol;
        P.error = err;
        long long total = 0;
        CK(cudaEventRecord(e0, c->stream));
        if (in->model == PICGPU_INIT_QUASINEUTRAL_PLASMA) {
            total = (long long)smp[sp].cell_count * nc;
        } else if (in->model == PICGPU_INIT_UNIFORM_DISPLACEMENT) {
            for (int a = 0; a < 3; ++a) {
                P.nl[a] = in->particle_numbers[a];
                P.lo[a] = lo[a];
                P.delta[a] = delta[a];
                P.dir[a] = dir[a];
                P.grid_lo[a] = glo[a];
                P.grid_hi[a] = ghi[a];
                P.grid_n[a] = m.n[a];
            }
            P.span_len = span_len;
            P.cycles = in->cycles;
            if (m.grid_cell.empty()) {
                release();
                return bad(c, PICGPU_NOT_SUPPORTED, "initialise: UniformDisplacement needs a block mesh");
            }
            total = in->particle_numbers[0] * in->particle_numbers[1] * in->particle_numbers[2];
        } else {
            pgd::launch_init_count(P, counts, c->stream);
            CK(pgd::init_scan(counts, offsets, sums, nc, c->stream));
            CK(cudaMemcpyAsync(&total, offsets + nc, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            c->launches += 4;
        }
        if ((ps = reserve_species(c, sp, total))) {
            release();
            return ps;
        }
        SpeciesBuf& B = c->sp[sp];
        P.first = B.n;
        P.tet = B.tet[B.cur];
        for (int a = 0; a < 3; ++a) {
            P.y64[a] = B.y64[B.cur][a];
            P.u64[a] = B.u64[B.cur][a];
            P.y32[a] = B.y32[B.cur][a];
            P.u32[a] = B.u32[B.cur][a];
        }
        if (in->model == PICGPU_INIT_UNIFORM_DISPLACEMENT) {
            const int* gc = nullptr;
            if ((ps = upload(c, const_cast<int**>(&gc), m.grid_cell))) {
                release();
                return ps;
            }
            P.grid_cell = gc;
            pgd::launch_init_fill_lattice(P, c->stream);
            CK(cudaStreamSynchronize(c->stream));
            dfree(c, const_cast<int*>(gc));
        } else if (in->model == PICGPU_INIT_QUASINEUTRAL_PLASMA) {
            pgd::launch_init_fill_cells(P, c->stream);
        } else {
            pgd::launch_init_fill_tets(P, offsets, c->stream);
        }
        c->launches++;
        CK(cudaEventRecord(e1, c->stream));
        int e = 0;
        CK(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaGetLastError());
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        place_ms += ms;
        if (e) {
            release();
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return bad(c, e == 2 ? PICGPU_CAPACITY : PICGPU_INVALID_ARG,
                       e == 2 ? "initialise: more than 2^24 particles in one tet"
                              : "initialise: tried to create a particle outside of the mesh");
        }
        pgd::launch_fill_attributes(view(c, sp, B.cur), B.n, B.n + total, c->cfg.species[sp].weight, c->stream);
        B.n += total;
        B.alive += total;
        S.added[sp] = total;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    S.place_ms = place_ms;

    // statistics (picInitialise.C:86-188)
    double vol = 0, lsum = 0;
    for (int k = 0; k < nc; ++k) {
        vol += m.vol[k];
        lsum += std::cbrt(m.vol[k]);
    }
    S.mesh_volume = vol;
    S.average_cell_size = nc > 0 ? lsum / nc : 0.0;
    for (int sp = 0; sp < ns; ++sp) {
        const SpeciesBuf& B = c->sp[sp];
        const picgpu_species& P = c->cfg.species[sp];
        pgd::launch_init_occupancy(B.tet[B.cur], B.n, nc, counts, c->stream);
        pgd::launch_init_minmax(counts, nc, mm, c->stream);
        long long h[3];
        CK(cudaMemcpyAsync(h, mm, sizeof h, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemsetAsync(c->diag, 0, 10 * sizeof(double), c->stream));
        const pgd::DSpecies v = view(c, sp, B.cur);
        pgd::launch_diagnostics(v.tet, v.u64[0], v.u64[1], v.u64[2], v.u32[0], v.u32[1], v.u32[2], int(B.n),
                                P.mass, P.weight, v.nw, c->diag, c->stream);
        double d[10];
        CK(cudaMemcpyAsync(d, c->diag, sizeof d, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->launches += 3;
        S.occupancy_min[sp] = h[0];
        S.occupancy_max[sp] = h[1];
        S.occupancy_avg[sp] = nc > 0 ? double(h[2]) / nc : 0.0;
        const double N = d[8];  // sum of nParticle
        if (N > 0) {
            double v2 = 0, dd = 0;
            for (int a = 0; a < 3; ++a) {
                S.drift[sp][a] = d[2 + a] / (P.mass * N);
                v2 += d[5 + a];
                dd += S.drift[sp][a] * S.drift[sp][a];
            }
            S.temperature[sp] = P.mass / (3.0 * kBoltzmann) * (v2 / N - dd);
        }
        S.number_density[sp] = vol > 0 ? N / vol : 0.0;
        S.model_temperature[sp] = calc_T ? S.temperature[sp] : in->temperature[sp];
        S.model_number_density[sp] = calc_n ? S.number_density[sp] : in->number_density[sp];
    }
    {
        const double eps0 = 1.0 / (kMu0 * kCl * kCl);
        double inv_l2 = 0;
        for (int sp = 0; sp < ns; ++sp) {
            const double q = c->cfg.species[sp].charge;
            const double T = S.model_temperature[sp], n = S.model_number_density[sp];
            if (q == 0.0 || n <= 0.0 || T <= 0.0) continue;
            inv_l2 += n * q * q / eps0 / (T * kBoltzmann);
        }
        S.debye_length = inv_l2 > 0 ? std::sqrt(1.0 / inv_l2) : 0.0;
        const int el = c->cfg.electron_species;
        if (el >= 0 && el < ns && S.model_number_density[el] > 0) {
            const double q = c->cfg.species[el].charge;
            S.plasma_frequency_dt =
                std::sqrt(S.model_number_density[el] * q * q / eps0 / c->cfg.species[el].mass) * c->cfg.dt;
        }
    }
    release();

    // calculateFields, solveMaxwellEquations (picInitialise.C:209-217)
    if ((ps = zero_accumulators(c)) || (ps = move_species(c, true)) || (ps = charge_update(c))) return ps;
    if (in->solve_fields && (ps = solve_fields(c, nullptr))) return ps;
    // initalizeLeapFrog (picInitialise.C:219-227)
    if (in->leapfrog) {
        for (int sp = 0; sp < ns; ++sp) {
            if (c->sp[sp].n == 0) continue;
            pgd::MoveParams P = move_params(c, sp, false);
            pgd::launch_push_only(P, c->mixed, -0.5 * c->cfg.dt, grid_for(c, c->sp[sp].n), c->stream);
            c->launches++;
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    if (c->profiling) harvest_events(c);
    if (st) *st = S;
    (void)kElementary;
    return PICGPU_OK;
}

picgpu_status picgpu_step(picgpu_ctx* c, int nsteps, picgpu_step_stats* stats) {
    if (!c || nsteps < 0) return PICGPU_INVALID_ARG;
    if (stats) std::memset(stats, 0, sizeof *stats);
    for (int k = 0; k < nsteps; ++k) {
        picgpu_status s = one_step(c, stats, true);
        if (s) return s;
    }
    if (c->profiling) harvest_events(c);
    fill_counts(c, stats);
    if (stats) {
        std::vector<double> sg(c->m.patches.size());
        CK(cudaMemcpy(sg.data(), c->sigma, sg.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t p = 0; p < sg.size() && p < PICGPU_MAX_BOXES + 6; ++p)
            stats->floating_charge[p] = sg[p] * c->m.patches[p].area;
        if (c->circ_state) {
            pg::CircuitState cs;
            CK(cudaMemcpy(&cs, c->circ_state, sizeof cs, cudaMemcpyDeviceToHost));
            stats->circuit_voltage = cs.voltage;
            stats->circuit_current = cs.current;
            stats->circuit_cathode_current = cs.cathode_current;
            stats->circuit_charge = cs.charge;
        }
    }
    return PICGPU_OK;
}

picgpu_status picgpu_move(picgpu_ctx* c, picgpu_step_stats* stats) {
    if (!c) return PICGPU_INVALID_ARG;
    if (stats) std::memset(stats, 0, sizeof *stats);
    picgpu_status s = one_step(c, stats, false);
    if (s) return s;
    CK(cudaStreamSynchronize(c->stream));
    if (c->profiling) harvest_events(c);
    fill_counts(c, stats);
    return PICGPU_OK;
}

picgpu_status picgpu_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return PICGPU_INVALID_ARG;
    *ptr = nullptr;
    if (bytes == 0) return PICGPU_OK;
    if (cudaMallocHost(ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return PICGPU_OOM;
    }
    return PICGPU_OK;
}

picgpu_status picgpu_host_free(void* ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return PICGPU_INVALID_ARG;
    }
    return PICGPU_OK;
}

picgpu_status picgpu_solve_poisson(picgpu_ctx* c, const double* rho, double* phi_inout,
                                   picgpu_step_stats* stats) {
    if (!c || !rho || !phi_inout) return PICGPU_INVALID_ARG;
    if (stats) std::memset(stats, 0, sizeof *stats);
    const size_t n = c->m.n_cells;
    CK(cudaMemcpyAsync(c->rho, rho, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->phi, phi_inout, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    picgpu_status s = poisson(c, stats);
    CK(cudaMemcpyAsync(phi_inout, c->phi, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (c->profiling) harvest_events(c);
    return s;
}

picgpu_status picgpu_upload_particles(picgpu_ctx* c, const picgpu_particles_soa* p, size_t n) {
    if (!c || !p || (n > 0 && (!p->species || !p->tet || !p->bary || !p->U))) return PICGPU_INVALID_ARG;
    const int ns = c->cfg.n_species;
    std::vector<std::vector<size_t>> idx(ns);
    for (size_t i = 0; i < n; ++i) {
        const int s = p->species[i];
        if (s < 0 || s >= ns) return bad(c, PICGPU_INVALID_ARG, "upload_particles: species out of range");
        idx[s].push_back(i);
    }
    std::vector<int32_t> tet;
    std::vector<double> bary, U;
    for (int s = 0; s < ns; ++s) {
        const size_t m = idx[s].size();
        tet.resize(m);
        bary.resize(3 * m);
        U.resize(3 * m);
        for (size_t k = 0; k < m; ++k) {
            const size_t i = idx[s][k];
            tet[k] = p->tet[i];
            for (int a = 0; a < 3; ++a) {
                bary[3 * k + a] = p->bary[3 * i + a];
                U[3 * k + a] = p->U[3 * i + a];
            }
        }
        picgpu_status st = picgpu_set_particles(c, s, m, tet.data(), bary.data(), U.data());
        if (st) return st;
    }
    return PICGPU_OK;
}

picgpu_status picgpu_download_particles(picgpu_ctx* c, picgpu_particles_soa* p, size_t cap, size_t* n) {
    if (!c || !p || !n) return PICGPU_INVALID_ARG;
    size_t total = 0;
    std::vector<size_t> cnt(c->cfg.n_species);
    for (int s = 0; s < c->cfg.n_species; ++s) {
        picgpu_status st = picgpu_count_particles(c, s, &cnt[s]);
        if (st) return st;
        total += cnt[s];
    }
    *n = total;
    if (total > cap) return bad(c, PICGPU_INVALID_ARG, "download_particles: the buffers are too small");
    if (total > 0 && (!p->species || !p->tet || !p->bary || !p->U)) return PICGPU_INVALID_ARG;
    size_t at = 0;
    for (int s = 0; s < c->cfg.n_species; ++s) {
        size_t got = 0;
        picgpu_status st =
            picgpu_get_particles(c, s, cap - at, p->tet + at, p->bary + 3 * at, p->U + 3 * at, &got);
        if (st) return st;
        for (size_t k = 0; k < got; ++k) p->species[at + k] = s;
        at += got;
    }
    *n = at;
    return PICGPU_OK;
}

picgpu_status picgpu_get_fields(picgpu_ctx* c, double* phi, double* E, double* rho) {
    if (!c) return PICGPU_INVALID_ARG;
    const size_t nc = c->m.n_cells;
    picgpu_status st;
    if (phi && (st = picgpu_get_field(c, PICGPU_FIELD_PHI, phi, nc))) return st;
    if (E && (st = picgpu_get_field(c, PICGPU_FIELD_E_CELL, E, 3 * nc))) return st;
    if (rho && (st = picgpu_get_field(c, PICGPU_FIELD_RHO, rho, nc))) return st;
    return PICGPU_OK;
}

picgpu_status picgpu_get_field(picgpu_ctx* c, int which, double* out, size_t n) {
    if (!c || !out) return PICGPU_INVALID_ARG;
    const double* src = nullptr;
    size_t cnt = 0;
    switch (which) {
        case PICGPU_FIELD_PHI: src = c->phi; cnt = c->m.n_cells; break;
        case PICGPU_FIELD_E_CELL: src = c->E; cnt = 3 * size_t(c->m.n_cells); break;
        case PICGPU_FIELD_RHO: src = c->rho; cnt = c->m.n_cells; break;
        case PICGPU_FIELD_E_POINT: src = c->Ept; cnt = 3 * size_t(c->m.n_points); break;
        case PICGPU_FIELD_SIGMA_V_MAX:
            src = c->coll.svmax;
            cnt = c->m.n_cells;
            if (!src) return bad(c, PICGPU_INVALID_ARG, "no MCC state");
            break;
        case PICGPU_FIELD_PATCH_SIGMA: {
            const size_t np = c->m.patches.size();
            if (n < np) return bad(c, PICGPU_INVALID_ARG, "output buffer too small");
            std::vector<double> sg(np);
            CK(cudaStreamSynchronize(c->stream));
            CK(cudaMemcpy(sg.data(), c->sigma, np * sizeof(double), cudaMemcpyDeviceToHost));
            for (size_t p = 0; p < np; ++p) out[p] = c->m.patches[p].p.kind == PICGPU_PATCH_FLOATING ? sg[p] : 0.0;
            return PICGPU_OK;
        }
        case PICGPU_FIELD_B_CELL:
            src = c->Bc;
            cnt = 3 * size_t(c->m.n_cells);
            if (!src) {
                if (n < cnt) return bad(c, PICGPU_INVALID_ARG, "output buffer too small");
                for (size_t k = 0; k < cnt; ++k) out[k] = c->cfg.B[k % 3];
                return PICGPU_OK;
            }
            break;
        default: return PICGPU_INVALID_ARG;
    }
    if (n < cnt) return bad(c, PICGPU_INVALID_ARG, "output buffer too small");
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(out, src, cnt * sizeof(double), cudaMemcpyDeviceToHost));
    return PICGPU_OK;
}

picgpu_status picgpu_set_field(picgpu_ctx* c, int which, const double* in, size_t n) {
    if (!c || !in) return PICGPU_INVALID_ARG;
    if (which == PICGPU_FIELD_PATCH_SIGMA) {
        const size_t np = c->m.patches.size();
        if (n < np) return bad(c, PICGPU_INVALID_ARG, "input buffer too small");
        std::vector<double> sg(np);
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaMemcpy(sg.data(), c->sigma, np * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t p = 0; p < np; ++p)
            if (c->m.patches[p].p.kind == PICGPU_PATCH_FLOATING) sg[p] = in[p];
        CK(cudaMemcpy(c->sigma, sg.data(), np * sizeof(double), cudaMemcpyHostToDevice));
        // the floating update with an empty accumulator: gradient sigma / eps0
        pgd::launch_floating_update(c->qconv, c->sigma, c->grad_bc, c->stream);
        c->launches++;
        CK(cudaStreamSynchronize(c->stream));
        return PICGPU_OK;
    }
    if (which == PICGPU_FIELD_B_CELL) {
        const size_t nb = 3 * size_t(c->m.n_cells);
        if (n < nb) return bad(c, PICGPU_INVALID_ARG, "input buffer too small");
        if (c->n_cases > 1 || !c->graphs.empty())
            return bad(c, PICGPU_NOT_SUPPORTED, "a per-cell magnetic field is not supported with ensembles or graph steps");
        picgpu_status st;
        if (!c->Bc && ((st = dalloc(c, &c->Bc, nb)) || (st = dalloc(c, &c->Bc4, size_t(c->m.n_cells))))) return st;
        std::vector<float4> b4(c->m.n_cells);
        bool any = false;
        for (size_t k = 0; k < size_t(c->m.n_cells); ++k) {
            b4[k] = make_float4(float(in[3 * k]), float(in[3 * k + 1]), float(in[3 * k + 2]), 0.f);
            any = any || in[3 * k] != 0.0 || in[3 * k + 1] != 0.0 || in[3 * k + 2] != 0.0;
        }
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaMemcpy(c->Bc, in, nb * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->Bc4, b4.data(), b4.size() * sizeof(float4), cudaMemcpyHostToDevice));
        // the pushers skip the rotation only when B vanishes everywhere (BorisPusher.C:43-55)
        c->rotation = any;
        return PICGPU_OK;
    }
    double* dst = nullptr;
    size_t cnt = 0;
    switch (which) {
        case PICGPU_FIELD_PHI: dst = c->phi; cnt = c->m.n_cells; break;
        case PICGPU_FIELD_E_CELL: dst = c->E; cnt = 3 * size_t(c->m.n_cells); break;
        case PICGPU_FIELD_RHO: dst = c->rho; cnt = c->m.n_cells; break;
        case PICGPU_FIELD_E_POINT: dst = c->Ept; cnt = 3 * size_t(c->m.n_points); break;
        default: return PICGPU_INVALID_ARG;
    }
    if (n < cnt) return bad(c, PICGPU_INVALID_ARG, "input buffer too small");
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(dst, in, cnt * sizeof(double), cudaMemcpyHostToDevice));
    pgd::launch_to_float(c->E, c->E32, 3L * c->m.n_cells, c->stream);
    pgd::launch_to_float(c->Ept, c->Ept32, 3L * c->m.n_points, c->stream);
    c->launches += 2;
    if (c->Ec4) {
        pgd::launch_corner_E(c->dm, c->E, c->Ept, c->Ec4, c->stream);
        c->launches++;
    }
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_diagnostics_compute(picgpu_ctx* c, picgpu_diagnostics* out) {
    if (!c || !out) return PICGPU_INVALID_ARG;
    std::memset(out, 0, sizeof *out);
    CK(cudaMemsetAsync(c->diag, 0, 64 * sizeof(double), c->stream));
    for (int s = 0; s < c->cfg.n_species; ++s) {
        const SpeciesBuf& B = c->sp[s];
        pgd::launch_diagnostics(B.tet[B.cur], c->mixed ? nullptr : B.u64[B.cur][0],
                                c->mixed ? nullptr : B.u64[B.cur][1], c->mixed ? nullptr : B.u64[B.cur][2],
                                B.u32[B.cur][0], B.u32[B.cur][1], B.u32[B.cur][2], int(B.n),
                                c->cfg.species[s].mass, c->cfg.species[s].weight,
                                B.attrs ? B.nw[B.cur] : nullptr, c->diag + 10 * s, c->stream);
        c->launches++;
    }
    pgd::launch_field_energy(c->E, c->dm.vol, c->m.n_cells, c->diag + 60, c->stream);
    c->launches++;
    double h[64];
    CK(cudaMemcpyAsync(h, c->diag, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int s = 0; s < c->cfg.n_species; ++s) {
        const double* v = h + 10 * s;
        out->kinetic_energy[s] = v[0];
        out->kinetic_energy_rel[s] = v[1];
        for (int a = 0; a < 3; ++a) {
            out->momentum[s][a] = v[2 + a];
            out->velocity_sq[s][a] = v[5 + a];
        }
        out->weight_sum[s] = v[8];
    }
    const double eps0 = 1.0 / (kMu0 * kCl * kCl);
    out->field_energy = 0.5 * eps0 * h[60];
    return PICGPU_OK;
}

picgpu_status picgpu_set_profiling(picgpu_ctx* c, int enabled) {
    if (!c) return PICGPU_INVALID_ARG;
    c->profiling = enabled != 0;
    return PICGPU_OK;
}

picgpu_status picgpu_phase_times(picgpu_ctx* c, double* ms, int64_t* launches, int nphase, int reset) {
    if (!c) return PICGPU_INVALID_ARG;
    CK(cudaStreamSynchronize(c->stream));
    harvest_events(c);
    for (int i = 0; i < nphase && i < PICGPU_PHASE_COUNT; ++i) {
        if (ms) ms[i] = c->phase_ms[i];
        if (launches) launches[i] = c->phase_launches[i];
    }
    if (reset)
        for (int i = 0; i < PICGPU_PHASE_COUNT; ++i) { c->phase_ms[i] = 0; c->phase_launches[i] = 0; }
    return PICGPU_OK;
}

int64_t picgpu_kernel_launches(const picgpu_ctx* c) { return c ? c->launches : 0; }

picgpu_status picgpu_synchronize(picgpu_ctx* c) {
    if (!c) return PICGPU_INVALID_ARG;
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_timer_start(picgpu_ctx* c) {
    if (!c) return PICGPU_INVALID_ARG;
    if (!c->timer[0]) {
        CK(cudaEventCreate(&c->timer[0]));
        CK(cudaEventCreate(&c->timer[1]));
    }
    CK(cudaEventRecord(c->timer[0], c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_timer_stop(picgpu_ctx* c, double* ms) {
    if (!c || !ms || !c->timer[0]) return PICGPU_INVALID_ARG;
    CK(cudaEventRecord(c->timer[1], c->stream));
    CK(cudaEventSynchronize(c->timer[1]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, c->timer[0], c->timer[1]));
    *ms = f;
    return PICGPU_OK;
}

}  // extern "C"

// ------------------------------------------------------------ ensembles --
extern "C" {

picgpu_status picgpu_ensemble_set_efield(picgpu_ctx* c, const double* E) {
    if (!c || !E) return PICGPU_INVALID_ARG;
    if (c->cfg.maxwell_solver != PICGPU_MAXWELL_NONE)
        return bad(c, PICGPU_INVALID_ARG, "ensemble E field: MaxwellSolver must be none");
    const long nc = c->m.n_cells / c->n_cases, np = c->m.n_points / c->n_cases;
    std::vector<double> e(3 * size_t(c->m.n_cells)), ep(3 * size_t(c->m.n_points));
    for (long i = 0; i < c->m.n_cells; ++i)
        for (int a = 0; a < 3; ++a) e[3 * i + a] = E[3 * (i / nc) + a];
    for (long i = 0; i < c->m.n_points; ++i)
        for (int a = 0; a < 3; ++a) ep[3 * i + a] = E[3 * (i / np) + a];
    CK(cudaMemcpyAsync(c->E, e.data(), e.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->Ept, ep.data(), ep.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    pgd::launch_to_float(c->E, c->E32, long(e.size()), c->stream);
    pgd::launch_to_float(c->Ept, c->Ept32, long(ep.size()), c->stream);
    c->launches += 2;
    if (c->Ec4) {
        pgd::launch_corner_E(c->dm, c->E, c->Ept, c->Ec4, c->stream);
        c->launches++;
    }
    CK(cudaStreamSynchronize(c->stream));
    return PICGPU_OK;
}

picgpu_status picgpu_ensemble_case_stats(picgpu_ctx* c, int species, double* out, int64_t* ionisations) {
    if (!c || !out || species < 0 || species >= c->cfg.n_species) return PICGPU_INVALID_ARG;
    const int cases = c->n_cases;
    const int cpc = c->m.n_cells / cases;
    double* d = nullptr;
    CK(cudaMalloc(&d, sizeof(double) * 5 * cases));
    CK(cudaMemsetAsync(d, 0, sizeof(double) * 5 * cases, c->stream));
    const SpeciesBuf& B = c->sp[species];
    const pgd::DSpecies v = view(c, species, B.cur);
    const int grid = std::max(1, std::min<int>(int((B.n + 255) / 256), 4 * c->sm_count));
    const size_t sm = sizeof(double) * 5 * cases;
    if (B.n > 0) {
        if (c->mixed)
            case_stats_kernel<float><<<grid, 256, sm, c->stream>>>(v.tet, v.u32[0], v.u32[1], v.u32[2], B.n, cpc,
                                                                    cases, d);
        else
            case_stats_kernel<double><<<grid, 256, sm, c->stream>>>(v.tet, v.u64[0], v.u64[1], v.u64[2], B.n, cpc,
                                                                     cases, d);
    }
    cudaError_t e = cudaMemcpyAsync(out, d, sizeof(double) * 5 * cases, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && ionisations) {
        if (c->coll.iz_cell) {
            unsigned long long* di = nullptr;
            e = cudaMalloc(&di, sizeof(unsigned long long) * cases);
            if (e == cudaSuccess) {
                case_sum_kernel<<<cases, 256, 0, c->stream>>>(c->coll.iz_cell, cpc, di);
                e = cudaMemcpyAsync(ionisations, di, sizeof(int64_t) * cases, cudaMemcpyDeviceToHost, c->stream);
                cudaStreamSynchronize(c->stream);
                cudaFree(di);
            }
        } else {
            for (int k = 0; k < cases; ++k) ionisations[k] = 0;
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    CK(e);
    return PICGPU_OK;
}

picgpu_status picgpu_step_graph(picgpu_ctx* c, int nsteps, int steps_per_graph, picgpu_step_stats* stats) {
    if (c && (!c->injectors.empty() || !c->freestreams.empty() || !c->emitters.empty()))
        return bad(c, PICGPU_NOT_SUPPORTED, "step_graph: injection runs only in picgpu_step");
    if (c && c->circ.model != PICGPU_CIRCUIT_NONE)
        return bad(c, PICGPU_NOT_SUPPORTED, "step_graph: circuit models run only in picgpu_step");
    if (c && ((c->cfg.mcc.enabled && c->cfg.mcc.neutral_parcels) ||
              (c->cfg.ion_mcc.enabled && c->cfg.ion_mcc.neutral_parcels)))
        return bad(c, PICGPU_NOT_SUPPORTED, "step_graph: collisions with neutral parcels run only in picgpu_step");
    if (!c || nsteps < 0 || steps_per_graph <= 0 || nsteps % steps_per_graph) return PICGPU_INVALID_ARG;
    if (!c->mixed || c->cfg.maxwell_solver != PICGPU_MAXWELL_NONE)
        return bad(c, PICGPU_NOT_SUPPORTED, "graph steps need the FP32 form and MaxwellSolver none");
    if (stats) *stats = picgpu_step_stats{};
    int replays = nsteps / steps_per_graph;
    picgpu_status s;
    if (!c->tuned && replays > 0) {
        // autotune on live steps (the physics does not depend on the launch
        // shape: per-particle moves, integer deposits, per-cell collisions):
        // two replays per candidate, the second one timed and normalised by
        // the particles it moved (the population changes while tuning)
        const int bps_cand[] = {3, 4, 5, 6, 8};
        const int mcc_cand[] = {64, 128, 256};
        c->tune_ms.clear();
        int best_bps = c->move_bps, best_mcc = c->coll.mcc_block;
        double best = 1e30;
        for (int b : bps_cand) {
            if (replays < 2) break;
            c->move_bps = b;
            float ms = 0.f;
            if ((s = graph_replay(c, steps_per_graph, stats, nullptr))) return s;
            const double n0 = double(total_particles(c));
            if ((s = graph_replay(c, steps_per_graph, stats, &ms))) return s;
            const double per = ms / (0.5 * (n0 + double(total_particles(c))) * steps_per_graph + 1.0);
            replays -= 2;
            c->tune_ms.push_back(1e6 * per);
            if (per < best) { best = per; best_bps = b; }
        }
        c->move_bps = best_bps;
        if (any_collisions(c) && c->cfg.mcc.enabled) {
            best = 1e30;
            for (int b : mcc_cand) {
                if (replays < 2) break;
                c->coll.mcc_block = b;
                float ms = 0.f;
                if ((s = graph_replay(c, steps_per_graph, stats, nullptr))) return s;
                const double n0 = double(total_particles(c));
                if ((s = graph_replay(c, steps_per_graph, stats, &ms))) return s;
                const double per = ms / (0.5 * (n0 + double(total_particles(c))) * steps_per_graph + 1.0);
                replays -= 2;
                c->tune_ms.push_back(1e6 * per);
                if (per < best) { best = per; best_mcc = b; }
            }
            c->coll.mcc_block = best_mcc;
        }
        c->tuned = true;
    }
    for (int r = 0; r < replays; ++r)
        if ((s = graph_replay(c, steps_per_graph, stats, nullptr))) return s;
    if (c->profiling) harvest_events(c);
    fill_counts(c, stats);
    return PICGPU_OK;
}

picgpu_status picgpu_graph_tuning(picgpu_ctx* c, int* move_blocks_per_sm, int* mcc_block, double* times,
                                  int n_times) {
    if (!c) return PICGPU_INVALID_ARG;
    if (move_blocks_per_sm) *move_blocks_per_sm = c->move_bps;
    if (mcc_block) *mcc_block = c->coll.mcc_block;
    for (int k = 0; times && k < n_times; ++k) times[k] = k < int(c->tune_ms.size()) ? c->tune_ms[k] : 0.0;
    return PICGPU_OK;
}

}  // extern "C"
