// collide.cu -- collision step: cell occupancy, null-collision MCC, Coulomb.
//
//   cell occupancy   PICCloud::buildCellOccupancy (PICCloud.C:327-354): per
//                    species, the particle indices of every cell in storage
//                    order (counting sort + per-cell ordering by index, so the
//                    lists do not depend on atomic ordering)
//   mcc_*            ElectronNeutralCollisionModel::performBackgroundCollisions
//                    (submodels/CollisionModels/ElectronNeutralCollisionModel/
//                    ElectronNeutralCollisionModel/ElectronNeutralCollisionModel.C:703-829),
//                    one thread per cell, candidates drawn sequentially from a
//                    Philox stream keyed by (seed, cell, step); secondaries go
//                    to a staging slot per candidate and are appended in
//                    (cell, candidate) order; Nanbu or relativistic
//                    (RelativisticElectronNeutralCollision.C:161-242) scattering
//   ion_mcc_*        IonNeutralCollisionModel::performBackgroundCollisions
//                    (IonNeutralCollisionModel.C:453-577): isotropic elastic
//                    scattering or charge exchange, one thread per cell
//   coulomb_*        NanbuYonemuraPairing::pairANDcollide (NanbuYonemuraPairing.C:56-325)
//                    or TakizukaAbePairing::pairANDcollide (TakizukaAbePairing.C:60-341)
//                    with NanbuCollision::collide (NanbuCollision.C:60-161) or
//                    PerezRelativisticCollision::collide (PerezRelativisticCollision.C:60-220),
//                    fixed or Debye-length Coulomb logarithm
//                    (CoulombCollisionModel.C:249-309), one warp per cell
// The collision arithmetic is FP64 for both particle forms.
#include <algorithm>
#include <vector>

#include "collide.h"

namespace pgd {

__constant__ TetConst c_tetC;

namespace {

constexpr double kEch = 1.602176634e-19;
constexpr double kKb = 1.380649e-23;
constexpr double kPlanck = 6.62607015e-34;
constexpr double kMu0c = 4.0 * kPi * 1e-7;
__device__ __forceinline__ double eps0c() { return 1.0 / (kMu0c * kC * kC); }

// -------------------------------------------------------------- scans ---
__global__ void block_sums_kernel(const int* __restrict__ in, long n, int* __restrict__ sums) {
    __shared__ int ws[32];
    const long i = long(blockIdx.x) * 1024 + threadIdx.x;
    int v = i < n ? in[i] : 0;
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = ws[threadIdx.x];
        for (int off = 16; off >= 1; off >>= 1) w += __shfl_xor_sync(0xffffffffu, w, off);
        if (threadIdx.x == 0) sums[blockIdx.x] = w;
    }
}

// exclusive scan of sums[0..nb) in place, total into sums[nb]
__global__ void scan_sums_kernel(int* sums, int nb) {
    __shared__ int ws[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int x = v;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = ws[lane];
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            ws[lane] = w;
        }
        __syncthreads();
        const int incl = x + (warp > 0 ? ws[warp - 1] : 0);
        const int c0 = carry;
        if (i < nb) sums[i] = c0 + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void scan_apply_kernel(const int* __restrict__ in, long n, const int* __restrict__ sums,
                                  int* __restrict__ out) {
    __shared__ int ws[32];
    const long i = long(blockIdx.x) * 1024 + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int x = v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = ws[lane];
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        ws[lane] = w;
    }
    __syncthreads();
    const int incl = x + (warp > 0 ? ws[warp - 1] : 0);
    if (i < n) out[i] = sums[blockIdx.x] + incl - v;
    if (i == n - 1) out[n] = sums[blockIdx.x] + incl;
}

// out[0..n) exclusive prefix of in, out[n] = total; tmp needs n/1024 + 2 ints
void exclusive_scan(const int* in, int* out, long n, int* tmp, cudaStream_t s, int64_t* launches) {
    const long nb = (n + 1023) / 1024;
    block_sums_kernel<<<unsigned(nb), 1024, 0, s>>>(in, n, tmp);
    scan_sums_kernel<<<1, 1024, 0, s>>>(tmp, int(nb));
    scan_apply_kernel<<<unsigned(nb), 1024, 0, s>>>(in, n, tmp, out);
    *launches += 3;
}

// ---------------------------------------------------- cell occupancy -----
// The store is kept in cell order, so the lanes of a warp mostly share a
// cell: each group of lanes with one cell adds once (its leader), and in the
// scatter the lanes of a group take consecutive slots in lane order.  The
// warps step through the store together (whole warps in the loop).
__global__ void count_cells_kernel(const int32_t* __restrict__ tet, int n, int* __restrict__ count,
                                   const int* n_dev = nullptr) {
    if (n_dev) n = *n_dev;
    const int lane = threadIdx.x & 31;
    const long stride = long(gridDim.x) * blockDim.x;
    for (long w = long(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); w < n; w += stride) {
        const long i = w + lane;
        const int t = i < n ? tet[i] : -1;
        const int c = t >= 0 ? t / 12 : -1;
        const unsigned grp = __match_any_sync(0xffffffffu, c);
        if (c >= 0 && lane == __ffs(grp) - 1) atomicAdd(count + c, __popc(grp));
    }
}

__global__ void scatter_cells_kernel(const int32_t* __restrict__ tet, int n, const int* __restrict__ start,
                                     int* __restrict__ cursor, int* __restrict__ idx, const int* n_dev = nullptr) {
    if (n_dev) n = *n_dev;
    const int lane = threadIdx.x & 31;
    const long stride = long(gridDim.x) * blockDim.x;
    for (long w = long(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); w < n; w += stride) {
        const long i = w + lane;
        const int t = i < n ? tet[i] : -1;
        const int c = t >= 0 ? t / 12 : -1;
        const unsigned grp = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(grp) - 1;
        int b = 0;
        if (c >= 0 && lane == leader) b = atomicAdd(cursor + c, __popc(grp));
        b = __shfl_sync(0xffffffffu, b, leader);
        if (c >= 0) idx[start[c] + b + __popc(grp & ((1u << lane) - 1u))] = int(i);
    }
}

// Order every cell's list by particle index: one warp per cell; each lane
// ranks its element against the whole list through shuffles (indices are
// distinct), writes it to its rank in tmp, and the warp copies the list back.
// With `need`, only the cells whose need is non-zero (the background MCC's
// candidate counts, when nothing else reads the lists).
__global__ void order_cells_kernel(int n_cells, const int* __restrict__ start, int* __restrict__ idx,
                                   int* __restrict__ tmp, const int* __restrict__ need = nullptr) {
    const int cell = int((long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (cell >= n_cells) return;
    if (need && need[cell] == 0) return;
    const int s0 = start[cell];
    const int L = start[cell + 1] - s0;
    if (L <= 1) return;
    int* a = idx + s0;
    int* t = tmp + s0;
    // lists whose groups arrived in order are sorted already
    bool sorted = true;
    for (int i = lane + 1; i < L; i += 32) sorted = sorted && a[i - 1] < a[i];
    if (__all_sync(0xffffffffu, sorted)) return;
    if (L <= 64) {
        // bitonic network over 64 slots, element e = lane + 32 r in v[r]
        // (padding sorts last); pairs (e, e ^ j) hold (min, max) where
        // e & k == 0, (max, min) elsewhere
        int v[2] = {lane < L ? a[lane] : 0x7fffffff, lane + 32 < L ? a[lane + 32] : 0x7fffffff};
        for (int k = 2; k <= 64; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                if (j == 32) {
                    const int lo = min(v[0], v[1]), hi = max(v[0], v[1]);
                    const bool up = (lane & k) == 0;
                    v[0] = up ? lo : hi;
                    v[1] = up ? hi : lo;
                } else {
#pragma unroll
                    for (int r = 0; r < 2; ++r) {
                        const int e = lane + 32 * r;
                        const int w = __shfl_xor_sync(0xffffffffu, v[r], j);
                        const bool keep_min = ((e & j) == 0) == ((e & k) == 0);
                        v[r] = keep_min ? min(v[r], w) : max(v[r], w);
                    }
                }
            }
        }
        if (lane < L) a[lane] = v[0];
        if (lane + 32 < L) a[lane + 32] = v[1];
        return;
    }
    for (int base = 0; base < L; base += 32) {
        const int i = base + lane;
        const int v = i < L ? a[i] : 0x7fffffff;
        int rank = 0;
        for (int cb = 0; cb < L; cb += 32) {
            const int w = cb + lane < L ? a[cb + lane] : 0x7fffffff;
            const int m = min(32, L - cb);
            for (int k = 0; k < m; ++k) rank += __shfl_sync(0xffffffffu, w, k) < v ? 1 : 0;
        }
        if (i < L) t[rank] = v;
    }
    __syncwarp();
    for (int i = lane; i < L; i += 32) a[i] = t[i];
}

unsigned order_blocks(int n_cells) { return unsigned((long(n_cells) * 32 + 255) / 256); }

// ------------------------------------------------------------- Philox ---
struct Rng {
    Philox p;
    __device__ Rng(uint64_t seed, uint32_t stream, uint32_t cell, uint32_t step) : p(seed, stream, cell, step) {}
    __device__ double uniform() { return p.uniform(); }
    __device__ double normal() { return p.normal(); }
};

struct V3d { double x, y, z; };

template <class R> struct Vel;
template <> struct Vel<double> {
    static __device__ V3d get(const DSpecies& s, int i) { return {s.u64[0][i], s.u64[1][i], s.u64[2][i]}; }
    static __device__ void put(const DSpecies& s, int i, V3d v) { s.u64[0][i] = v.x; s.u64[1][i] = v.y; s.u64[2][i] = v.z; }
};
template <> struct Vel<float> {
    static __device__ V3d get(const DSpecies& s, int i) {
        return {double(s.u32[0][i]), double(s.u32[1][i]), double(s.u32[2][i])};
    }
    static __device__ void put(const DSpecies& s, int i, V3d v) {
        s.u32[0][i] = float(v.x); s.u32[1][i] = float(v.y); s.u32[2][i] = float(v.z);
    }
};

__device__ __forceinline__ double magd(V3d a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// Nanbu scattering (NanbuElectronNeutralCollision.C:97-131).
__device__ void nanbu_scatter(double eV, V3d& Ue, V3d& Un, double mE, double mN, Rng& r) {
    const double phi = 2.0 * kPi * r.uniform();
    double cosChi;
    if (eV < 1e-30) cosChi = 1.0;
    else cosChi = 1.0 / eV * (eV + 2.0 - 2.0 * pow(1.0 + eV, r.uniform()));
    double sinChi;
    if (cosChi * cosChi > 1.0) { cosChi = 1.0; sinChi = 0.0; }
    else sinChi = sqrt(1.0 - cosChi * cosChi);
    const V3d g = {Ue.x - Un.x, Ue.y - Un.y, Ue.z - Un.z};
    const double gm = magd(g);
    const double gp = sqrt(g.y * g.y + g.z * g.z);
    const double cp = cos(phi), sp = sin(phi);
    const V3d h = {gp * cp, -1.0 * (g.y * g.x * cp + gm * g.z * sp) / gp, -1.0 * (g.z * g.x * cp - gm * g.y * sp) / gp};
    const V3d d = {(1.0 - cosChi) * g.x + sinChi * h.x, (1.0 - cosChi) * g.y + sinChi * h.y,
                   (1.0 - cosChi) * g.z + sinChi * h.z};
    const double ke = mN / (mN + mE), kn = mE / (mN + mE);
    Ue = {Ue.x - ke * d.x, Ue.y - ke * d.y, Ue.z - ke * d.z};
    Un = {Un.x + kn * d.x, Un.y + kn * d.y, Un.z + kn * d.z};
}

__device__ __forceinline__ double dotd(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Centre-of-momentum frame of two particles and the rotation of the momentum
// in it (RelativisticElectronNeutralCollision.C:161-242,
// PerezRelativisticCollision.C:90-187).
struct CoM {
    double gP, gQ, gc, gcv, gPc, gQc, mag_pc;
    V3d vc, pc;
};

__device__ bool com_frame(V3d UP, V3d UQ, double mP, double mQ, CoM& f) {
    const double aP = magd(UP) / kC, aQ = magd(UQ) / kC;
    f.gP = 1.0 / sqrt(1.0 - aP * aP);
    f.gQ = 1.0 / sqrt(1.0 - aQ * aQ);
    const double kp = mP * f.gP, kq = mQ * f.gQ;
    const V3d pP = {kp * UP.x, kp * UP.y, kp * UP.z};
    const V3d pQ = {kq * UQ.x, kq * UQ.y, kq * UQ.z};
    const double den = mP * f.gP + mQ * f.gQ;
    f.vc = {(pP.x + pQ.x) / den, (pP.y + pQ.y) / den, (pP.z + pQ.z) / den};
    const double vc2 = dotd(f.vc, f.vc);
    if (vc2 == 0.0) {
        f.gc = 1.0;
        f.gcv = 0.5;
        f.pc = pP;
        f.gPc = f.gP;
        f.gQc = f.gQ;
    } else {
        f.gc = 1.0 / sqrt(1.0 - vc2 / (kC * kC));
        f.gcv = (f.gc - 1.0) / vc2;
        const double k = (f.gcv * dotd(f.vc, UP) - f.gc) * mP * f.gP;
        f.pc = {pP.x + k * f.vc.x, pP.y + k * f.vc.y, pP.z + k * f.vc.z};
        f.gPc = (1.0 - dotd(f.vc, UP) / (kC * kC)) * f.gP * f.gc;
        f.gQc = (1.0 - dotd(f.vc, UQ) / (kC * kC)) * f.gQ * f.gc;
    }
    f.mag_pc = magd(f.pc);
    return f.mag_pc != 0.0;
}

__device__ void com_rotate(const CoM& f, double cosChi, double sinChi, double eps, double mP, double mQ, V3d& UP,
                           V3d& UQ) {
    const double sce = sinChi * cos(eps), sse = sinChi * sin(eps);
    const V3d p = f.pc;
    const double pperp = sqrt(p.x * p.x + p.y * p.y);
    V3d np;
    if (pperp > 1.e-10 * f.mag_pc) {
        const double ip = 1.0 / pperp;
        np = {(p.x * p.z * sce - p.y * f.mag_pc * sse) * ip + p.x * cosChi,
              (p.y * p.z * sce + p.x * f.mag_pc * sse) * ip + p.y * cosChi, -pperp * sce + p.z * cosChi};
    } else {
        np = {f.mag_pc * sce, f.mag_pc * sse, f.mag_pc * cosChi};
    }
    const double kP = f.gcv * dotd(f.vc, np) + mP * f.gPc * f.gc;
    const V3d npP = {np.x + kP * f.vc.x, np.y + kP * f.vc.y, np.z + kP * f.vc.z};
    const double aP = magd(npP) / (mP * kC);
    const double ngP = sqrt(1.0 + aP * aP);
    const V3d mnp = {-1.0 * np.x, -1.0 * np.y, -1.0 * np.z};
    const double kQ = f.gcv * dotd(f.vc, mnp) + mQ * f.gQc * f.gc;
    const V3d npQ = {mnp.x + kQ * f.vc.x, mnp.y + kQ * f.vc.y, mnp.z + kQ * f.vc.z};
    const double aQ = magd(npQ) / (mQ * kC);
    const double ngQ = sqrt(1.0 + aQ * aQ);
    const double dP = mP * ngP, dQ = mQ * ngQ;
    UP = {npP.x / dP, npP.y / dP, npP.z / dP};
    UQ = {npQ.x / dQ, npQ.y / dQ, npQ.z / dQ};
}

// RelativisticElectronNeutralCollision::updateVelocity: cos(chi) is drawn
// before the azimuth.
__device__ void relativistic_scatter(double eV, V3d& Ue, V3d& Un, double mE, double mN, Rng& r) {
    CoM f;
    if (!com_frame(Ue, Un, mE, mN, f)) return;
    double cosChi;
    if (eV < 1e-30) cosChi = 1.0;
    else cosChi = 1.0 / eV * (eV + 2.0 - 2.0 * pow(1.0 + eV, r.uniform()));
    const double sinChi = sqrt(1.0 - cosChi * cosChi);
    const double eps = 2.0 * kPi * r.uniform();
    com_rotate(f, cosChi, sinChi, eps, mE, mN, Ue, Un);
}

__device__ __forceinline__ void electron_scatter(int relativistic, double eV, V3d& Ue, V3d& Un, double mE,
                                                 double mN, Rng& r) {
    if (relativistic) relativistic_scatter(eV, Ue, Un, mE, mN, r);
    else nanbu_scatter(eV, Ue, Un, mE, mN, r);
}

// List cross section, linear between bracketing nodes, end values held
// (ListCrossSection.C:33-88).  The tables of a collision model share one
// energy axis, so the bracket is searched once and every table read at it.
struct XsBracket {
    int lo, hi;
    int exact;   // -1 inside the bracket, else the node whose value is returned
};
__device__ XsBracket xs_bracket(double x, const double* e, int n) {
    if (x <= e[0]) return {0, 0, 0};
    if (x >= e[n - 1]) return {n - 1, n - 1, n - 1};
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] <= x) lo = mid; else hi = mid;
    }
    return {lo, hi, e[lo] == x ? lo : -1};
}
__device__ __forceinline__ double xs_at(const XsBracket& b, double x, const double* e, const double* v) {
    if (b.exact >= 0) return v[b.exact];
    return v[b.lo] + ((x - e[b.lo]) / (e[b.hi] - e[b.lo])) * (v[b.hi] - v[b.lo]);
}


__device__ __forceinline__ long mcc_candidates(const MccParams& M, int c, double* coll_out) {
    const int eC = M.e_start[c + 1] - M.e_start[c];
    const double coll = M.rem[c] + double(eC) * M.n_gas * M.svmax[c] * M.dt;
    *coll_out = coll;
    return eC > 0 ? long(coll) : 0;
}

__global__ void mcc_count_kernel(MccParams M, int* __restrict__ ncand) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    double coll;
    ncand[c] = int(mcc_candidates(M, c, &coll));
}

template <class R>
__global__ void mcc_kernel(MccParams M, DSpecies el, Secondary* __restrict__ stage) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    const int eC = M.e_start[c + 1] - M.e_start[c];
    const double sv = M.svmax[c];
    const double coll = M.rem[c] + double(eC) * M.n_gas * sv * M.dt;
    const long nC = long(coll);
    M.rem[c] = coll - double(nC);
    if (nC == 0 || eC == 0) return;
    const int* list = M.e_idx + M.e_start[c];
    const double* E = M.xs;
    const double* EL = M.xs + M.n_xs;
    const double* EX = M.xs + 2 * M.n_xs;
    const double* IZ = M.xs + 3 * M.n_xs;
    Rng r(M.seed, kStreamMcc, uint32_t(c), M.step_dev ? *M.step_dev : M.step);
    unsigned long long nel = 0, nex = 0, niz = 0;
    const int base = M.cand_off[c];
    const bool room = long(base) + nC <= M.stage_cap;
    if (!room) {
        // this cell's slots below the capacity stay unused: clear them so
        // that no stale flag is appended
        atomicExch(M.overflow, 1);
        for (long k = base; k < long(base) + nC && k < M.stage_cap; ++k) stage[k].flag = 0;
    }
    for (long i = 0; i < nC; ++i) {
        long j = long(r.uniform() * double(eC));
        if (j >= eC) j = eC - 1;
        const int pi = list[j];
        V3d Ue = Vel<R>::get(el, pi);
        const double n0 = r.normal(), n1 = r.normal(), n2 = r.normal();
        V3d Un = {M.vth_gas * n0 + M.drift[0], M.vth_gas * n1 + M.drift[1], M.vth_gas * n2 + M.drift[2]};
        const V3d d = {Ue.x - Un.x, Ue.y - Un.y, Ue.z - Un.z};
        const double cR = magd(d);
        const double gamma = 1.0 / sqrt(1.0 - (cR * cR) / (kC * kC));
        double eV = (gamma - 1.0) * M.me * kC * kC / kEch;
        const double sigmaT = sv / cR;
        const XsBracket xb = xs_bracket(eV, E, M.n_xs);
        const double Qel = xs_at(xb, eV, E, EL);
        const double Qex = xs_at(xb, eV, E, EX);
        const double Qiz = xs_at(xb, eV, E, IZ);
        const double Qt = Qel + Qex + Qiz;
        if (Qt * cR > M.svmax[c]) M.svmax[c] = Qt * cR;
        const double Ru = r.uniform();
        if (Ru <= Qel / sigmaT) {
            nel++;
            electron_scatter(M.relativistic, eV, Ue, Un, M.me, M.mg, r);
            Vel<R>::put(el, pi, Ue);
        } else if (eV >= M.ex_th && Ru <= (Qel + Qex) / sigmaT) {
            nex++;
            const double f = sqrt(1.0 - M.ex_th / eV);
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= M.ex_th;
            electron_scatter(M.relativistic, eV, Ue, Un, M.me, M.mg, r);
            Vel<R>::put(el, pi, Ue);
        } else if (eV >= M.iz_th && Ru <= Qt / sigmaT) {
            const double th = M.iz_th;
            const double E0 = 2.0 - 100.0 / (eV + 10.0);
            const double E1 = (eV - th) / 2.0 - E0;
            const double alpha = 10.3;
            const double Ep = E0 + alpha * tan(r.uniform() * (atan(E1 / alpha) + atan(E0 / alpha)) - atan(E0 / alpha));
            const V3d preUe = Ue;
            const V3d preUn = Un;
            const double f = sqrt(1.0 - (th + Ep) / eV);
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= (th + Ep);
            electron_scatter(M.relativistic, eV, Ue, Un, M.me, M.mg, r);
            const double rndU = r.uniform();
            Secondary sc{};
            const bool make = rndU <= M.wEwN;
            if (make && M.create_i) {
                sc.flag |= 2;
                sc.ui[0] = Un.x; sc.ui[1] = Un.y; sc.ui[2] = Un.z;
                niz++;
            }
            if (rndU > M.wNwE) Ue = preUe;
            Vel<R>::put(el, pi, Ue);
            if (make && M.create_e) {
                const double sp = sqrt(2.0 * Ep * kEch / M.me);
                const double mp = magd(preUe);
                V3d ne = {sp * (preUe.x / mp), sp * (preUe.y / mp), sp * (preUe.z / mp)};
                V3d un2 = preUn;
                electron_scatter(M.relativistic, Ep, ne, un2, M.me, M.mg, r);
                sc.flag |= 1;
                sc.ue[0] = ne.x; sc.ue[1] = ne.y; sc.ue[2] = ne.z;
            }
            if (sc.flag) {
                sc.tet = el.tet[pi];
                if (el.y64[0]) { sc.y[0] = el.y64[0][pi]; sc.y[1] = el.y64[1][pi]; sc.y[2] = el.y64[2][pi]; }
                else { sc.y[0] = el.y32[0][pi]; sc.y[1] = el.y32[1][pi]; sc.y[2] = el.y32[2][pi]; }
                sc.tet_i = sc.tet;
                for (int a = 0; a < 3; ++a) sc.y_i[a] = sc.y[a];
            }
            if (room) stage[base + i] = sc;
            continue;
        }
        if (room) stage[base + i].flag = 0;
    }
    if (M.iz_cell && niz) M.iz_cell[c] += niz;
    atomicAdd(M.counts + 0, (unsigned long long)nC);
    if (nel) atomicAdd(M.counts + 1, nel);
    if (nex) atomicAdd(M.counts + 2, nex);
    if (niz) atomicAdd(M.counts + 3, niz);
}

// ---------------------------------------------- neutral-parcel MCC -----
// ElectronNeutralCollisionModel::performCollisions
// (ElectronNeutralCollisionModel.C:833-1009): per cell, NTC candidates
// eC nC w_max (sigma_T c_R)_max dt / V, a random neutral parcel and a random
// electron per candidate, the running maximum updated, the events of the
// background model with the parcel's velocity as the partner
// (:489-645: the neutral takes its recoil unless updateNeutralVelocity is
// off; an ion is created at the neutral's position with its velocity, and
// the ionised neutral is deleted unless deleteNeutral is off).
struct MccParcelParams {
    int n_cells;
    const int* e_start;   // n_cells + 1
    const int* e_idx;
    const int* n_start;   // neutral species, n_cells + 1
    int* n_idx;           // its per-cell lists (deleted parcels are erased in place)
    double* svmax;
    double* rem;
    const double* vol;
    const double* xs;     // 4 x n_xs
    int n_xs;
    double me, mn, dt, wE, wN, wmax;
    double ex_th, iz_th;
    int create_e, create_i, relativistic, update_neutral, delete_neutral;
    uint64_t seed;
    uint32_t step;
    const int* cand_off;
    long stage_cap;
    int* overflow;
    unsigned long long* counts;
    int* n_live;          // per cell: neutral parcels left in the list at the end (read by the ion step)
};

__device__ __forceinline__ long parcel_candidates(const MccParcelParams& M, int c, double* sel) {
    const int eC = M.e_start[c + 1] - M.e_start[c];
    const int nC = M.n_start[c + 1] - M.n_start[c];
    const double sv = M.svmax[c];
    if (!(sv > 0.0) || nC == 0 || eC == 0) return 0;
    *sel = M.rem[c] + double(eC * nC) * M.wmax * sv * M.dt / M.vol[c];
    return long(*sel);
}

__global__ void mcc_parcel_count_kernel(MccParcelParams M, int* __restrict__ ncand) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    double sel = 0.0;
    ncand[c] = int(parcel_candidates(M, c, &sel));
}

template <class R>
__device__ __forceinline__ void stage_pos(const DSpecies& p, int i, int32_t& tet, double* y) {
    tet = p.tet[i];
    if (p.y64[0]) { y[0] = p.y64[0][i]; y[1] = p.y64[1][i]; y[2] = p.y64[2][i]; }
    else { y[0] = p.y32[0][i]; y[1] = p.y32[1][i]; y[2] = p.y32[2][i]; }
}

template <class R>
__global__ void mcc_parcel_kernel(MccParcelParams M, DSpecies el, DSpecies neu, Secondary* __restrict__ stage) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    double selected = 0.0;
    const long nCand = parcel_candidates(M, c, &selected);
    const int eC = M.e_start[c + 1] - M.e_start[c];
    int nC = M.n_start[c + 1] - M.n_start[c];
    M.n_live[c] = nC;
    const double sv = M.svmax[c];
    if (!(sv > 0.0) || nC == 0 || eC == 0) return;
    M.rem[c] = selected - double(nCand);
    if (nCand == 0) return;
    const int* elist = M.e_idx + M.e_start[c];
    int* nlist = M.n_idx + M.n_start[c];
    const double* E = M.xs;
    const double* EL = M.xs + M.n_xs;
    const double* EX = M.xs + 2 * M.n_xs;
    const double* IZ = M.xs + 3 * M.n_xs;
    Rng r(M.seed, kStreamMcc | 1u, uint32_t(c), M.step);
    unsigned long long nel = 0, nex = 0, niz = 0, ndel = 0, ncand = 0;
    const int base = M.cand_off[c];
    const bool room = long(base) + nCand <= M.stage_cap;
    if (!room) atomicExch(M.overflow, 1);
    long i = 0;
    for (; i < nCand; ++i) {
        ++ncand;
        long jn = long(r.uniform() * double(nC));
        if (jn >= nC) jn = nC - 1;
        long je = long(r.uniform() * double(eC));
        if (je >= eC) je = eC - 1;
        const int pn = nlist[jn], pe = elist[je];
        V3d Ue = Vel<R>::get(el, pe);
        V3d Un = Vel<R>::get(neu, pn);
        const V3d d = {Ue.x - Un.x, Ue.y - Un.y, Ue.z - Un.z};
        const double cR = magd(d);
        const double gamma = 1.0 / sqrt(1.0 - (cR * cR) / (kC * kC));
        double eV = (gamma - 1.0) * M.me * kC * kC / kEch;
        const XsBracket xb = xs_bracket(eV, E, M.n_xs);
        const double Qel = xs_at(xb, eV, E, EL);
        const double Qex = xs_at(xb, eV, E, EX);
        const double Qiz = xs_at(xb, eV, E, IZ);
        const double Qt = Qel + Qex + Qiz;
        if (Qt * cR > M.svmax[c]) M.svmax[c] = Qt * cR;
        const double rndU = r.uniform();
        Secondary sc{};
        if (rndU <= Qel * cR / sv) {
            nel++;
            electron_scatter(M.relativistic, eV, Ue, Un, M.me, M.mn, r);
            Vel<R>::put(el, pe, Ue);
            if (M.update_neutral) Vel<R>::put(neu, pn, Un);
        } else if (eV >= M.ex_th && rndU <= (Qel + Qex) * cR / sv) {
            nex++;
            const double f = sqrt(1.0 - M.ex_th / eV);
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= M.ex_th;
            electron_scatter(M.relativistic, eV, Ue, Un, M.me, M.mn, r);
            Vel<R>::put(el, pe, Ue);
            if (M.update_neutral) Vel<R>::put(neu, pn, Un);
        } else if (eV >= M.iz_th && rndU <= Qt * cR / sv) {
            const double th = M.iz_th;
            const double E0 = 2.0 - 100.0 / (eV + 10.0);
            const double E1 = (eV - th) / 2.0 - E0;
            const double alpha = 10.3;
            const double Ep = E0 + alpha * tan(r.uniform() * (atan(E1 / alpha) + atan(E0 / alpha)) - atan(E0 / alpha));
            const V3d preUe = Ue;
            const V3d preUn = Un;
            const double f = sqrt(1.0 - (th + Ep) / eV);
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= (th + Ep);
            const double wEwN = M.wE / M.wN, wNwE = 1.0 / wEwN;
            electron_scatter(M.relativistic, eV, Ue, Un, M.me, M.mn, r);
            const double rndU2 = r.uniform();
            bool created = false;
            if (rndU2 <= wEwN && M.create_i) {
                sc.flag |= 2;
                sc.ui[0] = Un.x; sc.ui[1] = Un.y; sc.ui[2] = Un.z;
                stage_pos<R>(neu, pn, sc.tet_i, sc.y_i);
                created = true;
            }
            if (rndU2 > wNwE) Ue = preUe;
            Vel<R>::put(el, pe, Ue);
            if (rndU2 <= wEwN && M.create_e) {
                const double sp = sqrt(2.0 * Ep * kEch / M.me);
                const double mp = magd(preUe);
                V3d ne = {sp * (preUe.x / mp), sp * (preUe.y / mp), sp * (preUe.z / mp)};
                V3d un2 = preUn;
                electron_scatter(M.relativistic, Ep, ne, un2, M.me, M.mn, r);
                sc.flag |= 1;
                sc.ue[0] = ne.x; sc.ue[1] = ne.y; sc.ue[2] = ne.z;
                stage_pos<R>(el, pe, sc.tet, sc.y);
            }
            if (M.update_neutral) Vel<R>::put(neu, pn, Un);
            if (created) {
                niz++;
                if (M.delete_neutral) {
                    neu.tet[pn] = -1;
                    for (long k = jn; k + 1 < nC; ++k) nlist[k] = nlist[k + 1];
                    --nC;
                    ++ndel;
                }
            }
        }
        if (room) stage[base + i] = sc;
        if (nC < 1) { ++i; break; }
    }
    if (room)
        for (; i < nCand; ++i) stage[base + i].flag = 0;   // candidates left after the last neutral went
    (void)ncand;
    // the ion - neutral parcel step reads this cell's list through the live
    // count: deleted neutrals were erased from it in place
    M.n_live[c] = nC;
    atomicAdd(M.counts + kCountMccParcel, (unsigned long long)nCand);
    if (nel) atomicAdd(M.counts + kCountMccParcel + 1, nel);
    if (nex) atomicAdd(M.counts + kCountMccParcel + 2, nex);
    if (niz) atomicAdd(M.counts + kCountMccParcel + 3, niz);
    if (ndel) atomicAdd(M.counts + 12, ndel);
}

// n_dev (optional): the staged count is read on the device; slots from it
// to n are flagged 0.
__global__ void stage_flags_kernel(const Secondary* __restrict__ stage, int n, int bit, int* __restrict__ flags,
                                   const int* n_dev = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int used = n_dev ? min(*n_dev, n) : n;
    if (i < n) flags[i] = (i < used && (stage[i].flag & bit)) ? 1 : 0;
}

// base_dev (optional): the destination offset is read on the device; slots
// at or beyond cap are dropped and raise *overflow.
template <class R>
__global__ void stage_append_kernel(const Secondary* __restrict__ stage, int n, int bit,
                                    const int* __restrict__ pos, DSpecies dst, int base,
                                    const int* base_dev = nullptr, long cap = 0, int* overflow = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(stage[i].flag & bit)) return;
    const long kk = long(base_dev ? *base_dev : base) + pos[i];
    if (base_dev && kk >= cap) {
        atomicExch(overflow, 1);
        return;
    }
    const int k = int(kk);
    const Secondary& s = stage[i];
    dst.tet[k] = bit == 1 ? s.tet : s.tet_i;
    const double* u = bit == 1 ? s.ue : s.ui;
    const double* y = bit == 1 ? s.y : s.y_i;
    if (dst.y64[0]) {
        for (int a = 0; a < 3; ++a) { dst.y64[a][k] = y[a]; dst.u64[a][k] = u[a]; }
    } else {
        for (int a = 0; a < 3; ++a) { dst.y32[a][k] = float(y[a]); dst.u32[a][k] = float(u[a]); }
    }
}

// IonNeutralCollisionModel::performCollisions (IonNeutralCollisionModel.C:
// 579-707) with the parcels of one neutral species: NTC candidates
// nC iC w_max (sigma_T c_R)_max dt / V per cell; IonIsotropicScattering of
// the pair (neutral P, ion Q; IonIsotropicScattering.C:60-100) or the
// charge-exchange identity switch with its weight gates (:401-413).
struct IonParcelParams {
    int n_cells;
    const int* i_start;
    const int* i_idx;
    const int* n_start;
    const int* n_idx;
    double* svmax;
    double* rem;
    const double* vol;
    const double* xs;     // 3 x n_xs: energy, elastic, charge exchange
    int n_xs;
    double mi, mn, dt, wI, wN, wmax, cx_th;
    int update_neutral;
    int weight_corr;      // PICGPU_WEIGHT_CORRECTION_* after an elastic scatter
    uint64_t seed;
    uint32_t step;
    unsigned long long* counts;
    const int* n_live;    // when set: live neutral parcels per cell (the electron step erased the ionised ones)
};

__device__ void weight_correct_pair(int model, double wP, double wQ, double mP, double mQ, V3d preP, V3d preQ,
                                    V3d& UP, V3d& UQ, Rng& r);

template <class R>
__global__ void ion_parcel_kernel(IonParcelParams M, DSpecies ions, DSpecies neu) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    const int iC = M.i_start[c + 1] - M.i_start[c];
    const int nC = M.n_live ? M.n_live[c] : M.n_start[c + 1] - M.n_start[c];
    if (nC == 0 || iC == 0) return;
    const double sv = M.svmax[c];
    const double selected = M.rem[c] + double(nC * iC) * M.wmax * sv * M.dt / M.vol[c];
    const long nCand = long(selected);
    M.rem[c] = selected - double(nCand);
    if (nCand == 0) return;
    const int* ilist = M.i_idx + M.i_start[c];
    const int* nlist = M.n_idx + M.n_start[c];
    const double* E = M.xs;
    const double* EL = M.xs + M.n_xs;
    const double* CX = M.xs + 2 * M.n_xs;
    Rng r(M.seed, kStreamIonMcc | 1u, uint32_t(c), M.step);
    unsigned long long nel = 0, ncx = 0;
    const double mt = M.mn + M.mi;
    for (long k = 0; k < nCand; ++k) {
        long jp = long(r.uniform() * double(nC));
        if (jp >= nC) jp = nC - 1;
        long jq = long(r.uniform() * double(iC));
        if (jq >= iC) jq = iC - 1;
        const int pp = nlist[jp], pq = ilist[jq];
        V3d UP = Vel<R>::get(neu, pp);
        V3d UQ = Vel<R>::get(ions, pq);
        const V3d d = {UQ.x - UP.x, UQ.y - UP.y, UQ.z - UP.z};
        const double cR = magd(d);
        const double gamma = 1.0 / sqrt(1.0 - (cR * cR) / (kC * kC));
        const double eV = (gamma - 1.0) * M.mi * kC * kC / kEch;
        const XsBracket xb = xs_bracket(eV, E, M.n_xs);
        const double Qel = xs_at(xb, eV, E, EL);
        const double Qcx = xs_at(xb, eV, E, CX);
        const double Qt = Qel + Qcx;
        if (Qt * cR > M.svmax[c]) M.svmax[c] = Qt * cR;
        const double rndU = r.uniform();
        if (rndU <= Qel * cR / sv) {
            nel++;
            const V3d preUP = UP;
            const V3d preUQ = UQ;
            const V3d Ucm = {(M.mn * UP.x + M.mi * UQ.x) / mt, (M.mn * UP.y + M.mi * UQ.y) / mt,
                             (M.mn * UP.z + M.mi * UQ.z) / mt};
            const V3d g = {UP.x - UQ.x, UP.y - UQ.y, UP.z - UQ.z};
            const double cr = magd(g);
            const double cosT = 2.0 * r.uniform() - 1.0;
            const double sinT = sqrt(1.0 - cosT * cosT);
            const double phi = 2.0 * kPi * r.uniform();
            const V3d rel = {cr * cosT, cr * (sinT * cos(phi)), cr * (sinT * sin(phi))};
            UP = {Ucm.x + rel.x * M.mi / mt, Ucm.y + rel.y * M.mi / mt, Ucm.z + rel.z * M.mi / mt};
            UQ = {Ucm.x - rel.x * M.mn / mt, Ucm.y - rel.y * M.mn / mt, Ucm.z - rel.z * M.mn / mt};
            // weightCorrection_->correctVelocity(pP, pQ, preUp, preUq) (:443-444)
            weight_correct_pair(M.weight_corr, M.wN, M.wI, M.mn, M.mi, preUP, preUQ, UP, UQ, r);
            if (!M.update_neutral) UP = preUP;
            Vel<R>::put(neu, pp, UP);
            Vel<R>::put(ions, pq, UQ);
        } else if (eV >= M.cx_th && rndU <= Qt * cR / sv) {
            ncx++;
            const double u = r.uniform();
            const V3d tmpP = UP;
            if (u <= M.wI / M.wN) UP = UQ;
            if (u <= M.wN / M.wI) UQ = tmpP;
            if (!M.update_neutral) UP = tmpP;
            Vel<R>::put(neu, pp, UP);
            Vel<R>::put(ions, pq, UQ);
        }
    }
    atomicAdd(M.counts + kCountIonParcel, (unsigned long long)nCand);
    if (nel) atomicAdd(M.counts + kCountIonParcel + 1, nel);
    if (ncx) atomicAdd(M.counts + kCountIonParcel + 2, ncx);
}

// --------------------------------------------------------- ion-neutral ---
struct IonMccParams {
    int n_cells;
    const int* i_start;   // n_cells + 1
    const int* i_idx;
    double* svmax;
    double* rem;
    const double* xs;     // 3 x n_xs: energy, elastic, charge exchange
    int n_xs;
    double n_gas, vth_gas, mg, mi, dt;
    double drift[3];
    double cx_th;
    uint64_t seed;
    uint32_t step;
    unsigned long long* counts;
    const unsigned* step_dev;
};

// IonNeutralCollisionModel::performBackgroundCollisions: elastic scattering
// isotropic in the centre-of-mass frame (IonIsotropicScattering.C:103-143) or
// charge exchange, the ion taking the neutral's velocity (:419-426).
template <class R>
__global__ void ion_mcc_kernel(IonMccParams M, DSpecies ions) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    const int nI = M.i_start[c + 1] - M.i_start[c];
    const double sv = M.svmax[c];
    const double coll = M.rem[c] + double(nI) * M.n_gas * sv * M.dt;
    const long nC = long(coll);
    M.rem[c] = coll - double(nC);
    if (nC == 0 || nI == 0) return;
    const int* list = M.i_idx + M.i_start[c];
    const double* E = M.xs;
    const double* EL = M.xs + M.n_xs;
    const double* CX = M.xs + 2 * M.n_xs;
    Rng r(M.seed, kStreamIonMcc, uint32_t(c), M.step_dev ? *M.step_dev : M.step);
    unsigned long long nel = 0, ncx = 0;
    const double mt = M.mi + M.mg;
    for (long i = 0; i < nC; ++i) {
        long j = long(r.uniform() * double(nI));
        if (j >= nI) j = nI - 1;
        const int pi = list[j];
        const V3d U = Vel<R>::get(ions, pi);
        const double n0 = r.normal(), n1 = r.normal(), n2 = r.normal();
        const V3d Un = {M.vth_gas * n0 + M.drift[0], M.vth_gas * n1 + M.drift[1], M.vth_gas * n2 + M.drift[2]};
        const V3d d = {U.x - Un.x, U.y - Un.y, U.z - Un.z};
        const double cR = magd(d);
        const double gamma = 1.0 / sqrt(1.0 - (cR * cR) / (kC * kC));
        const double eV = (gamma - 1.0) * M.mi * kC * kC / kEch;
        const double sigmaT = sv / cR;
        const XsBracket xb = xs_bracket(eV, E, M.n_xs);
        const double Qel = xs_at(xb, eV, E, EL);
        const double Qcx = xs_at(xb, eV, E, CX);
        const double Qt = Qel + Qcx;
        if (Qt * cR > M.svmax[c]) M.svmax[c] = Qt * cR;
        const double Ru = r.uniform();
        if (Ru <= Qel / sigmaT) {
            nel++;
            const V3d Ucm = {(M.mi * U.x + M.mg * Un.x) / mt, (M.mi * U.y + M.mg * Un.y) / mt,
                             (M.mi * U.z + M.mg * Un.z) / mt};
            const double cosT = 2.0 * r.uniform() - 1.0;
            const double sinT = sqrt(1.0 - cosT * cosT);
            const double phi = 2.0 * kPi * r.uniform();
            const V3d rel = {cR * cosT, cR * (sinT * cos(phi)), cR * (sinT * sin(phi))};
            Vel<R>::put(ions, pi,
                        V3d{Ucm.x + (M.mg * rel.x) / mt, Ucm.y + (M.mg * rel.y) / mt, Ucm.z + (M.mg * rel.z) / mt});
        } else if (eV >= M.cx_th && Ru <= Qt / sigmaT) {
            ncx++;
            Vel<R>::put(ions, pi, Un);
        }
    }
    atomicAdd(M.counts + 5, (unsigned long long)nC);
    if (nel) atomicAdd(M.counts + 6, nel);
    if (ncx) atomicAdd(M.counts + 7, ncx);
}

// ------------------------------------------------------------ Coulomb ---
struct CoulombSpecies {
    int n;                // charged species taking part
    int sp[PICGPU_MAX_SPECIES];
    double m[PICGPU_MAX_SPECIES], q[PICGPU_MAX_SPECIES], w[PICGPU_MAX_SPECIES];
    const int* start[PICGPU_MAX_SPECIES];
    const int* idx[PICGPU_MAX_SPECIES];
    int* sel[PICGPU_MAX_SPECIES];     // scratch permutation per species, same layout as idx
    int* sel2[PICGPU_MAX_SPECIES];
    DSpecies p[PICGPU_MAX_SPECIES];
};

// A parcel's nParticle and charge (species charge x chargeModifier,
// PICCloud.C:368): per parcel when the store has the arrays.
__device__ __forceinline__ double pweight(const CoulombSpecies& C, int k, int i) {
    return C.p[k].nw ? C.p[k].nw[i] : C.w[k];
}
__device__ __forceinline__ double pcharge(const CoulombSpecies& C, int k, int i) {
    return C.p[k].zq ? C.q[k] * double(C.p[k].zq[i]) : C.q[k];
}

__device__ double cos_chi(double s, Rng& r) {
    double U = r.uniform();
    if (s < 0.1) {
        if (U < 0.0001) U = 0.0001;
        return 1.0 + s * log(U);
    }
    if (s < 3.0) {
        const double invA = 0.00569578 + (0.95602 + (-0.508139 + (0.479139 + (-0.12789 + 0.0238957 * s) * s) * s) * s) * s;
        const double A = 1.0 / invA;
        return invA * log(exp(-A) + 2.0 * U * sinh(A));
    }
    if (s < 6.0) {
        const double A = 3.0 * exp(-s);
        return (1.0 / A) * log(exp(-A) + 2.0 * U * sinh(A));
    }
    return 2.0 * U - 1.0;
}

struct CoulombParams {
    int n_cells;
    const double* vol;
    double cl;            // fixed coulombLog; 0: from the cell Debye length
    int takizuka_abe;     // pairing: 0 NanbuYonemura, 1 TakizukaAbe
    int perez;            // collide: 0 Nanbu, 1 PerezRelativistic
    int allow_intra, calc_bmin, debye_drift, weight_corr;
    double dt;
    uint64_t seed;
    uint32_t step;
    unsigned long long* counts;
    const unsigned* step_dev;
};

// Sentoku-Kemp weight corrections: the parcel of the larger weight keeps the
// weight-averaged velocity (momentum) of before and after the collision
// plus a kick orthogonal to it that restores the weight-averaged kinetic
// (total) energy; the kick's azimuth is uniform.  Non-relativistic:
// SentokuKempNonRelCorrection.C:50-125; relativistic (momenta, total
// energies, Lorentz factors): SentokuKempCorrection.C:50-169.
__device__ void sk_basis(V3d a, double amag, V3d& e2, V3d& e3) {
    e2 = {0.0, 1.0, 0.0};
    e3 = {0.0, 0.0, 1.0};
    const double up = sqrt(a.y * a.y + a.z * a.z);
    if (up > 1.0e-300) {
        e2 = {0.0, a.z / up, -a.y / up};
        const double den = amag * up;
        e3 = {(up * up) / den, -(a.x * a.y) / den, -(a.x * a.z) / den};
    }
}

__device__ void sentoku_kemp_nr(double mass, double wr, V3d pre, V3d& U, Rng& r) {
    const V3d after = {(1.0 - wr) * pre.x + wr * U.x, (1.0 - wr) * pre.y + wr * U.y, (1.0 - wr) * pre.z + wr * U.z};
    const double afterE = (1.0 - wr) * 0.5 * mass * dotd(pre, pre) + wr * 0.5 * mass * dotd(U, U);
    const double dE = afterE - 0.5 * mass * dotd(after, after);
    if (!(dE > 0.0)) return;
    V3d e2, e3;
    sk_basis(after, sqrt(dotd(after, after)), e2, e3);
    const double eps = 6.283185307179586 * r.uniform();
    const double sp = sqrt(dE * 2.0 / mass), ce = cos(eps), se = sin(eps);
    U = {after.x + sp * (e2.x * ce + e3.x * se), after.y + sp * (e2.y * ce + e3.y * se),
         after.z + sp * (e2.z * ce + e3.z * se)};
}

__device__ void sentoku_kemp(double mass, double dw, V3d pre, V3d& U, Rng& r) {
    const double c = kC;
    const double mpre = sqrt(dotd(pre, pre)) / c, mpost = sqrt(dotd(U, U)) / c;
    const double g0 = 1.0 / sqrt(1.0 - mpre * mpre), g1 = 1.0 / sqrt(1.0 - mpost * mpost);
    const V3d p0 = {mass * g0 * pre.x, mass * g0 * pre.y, mass * g0 * pre.z};
    const V3d p1 = {mass * g1 * U.x, mass * g1 * U.y, mass * g1 * U.z};
    const double mc = mass * c;
    const double e0 = c * sqrt(dotd(p0, p0) + mc * mc), e1 = c * sqrt(dotd(p1, p1) + mc * mc);
    const double aE = (1.0 - dw) * e0 + dw * e1;
    const V3d aM = {(1.0 - dw) * p0.x + dw * p1.x, (1.0 - dw) * p0.y + dw * p1.y, (1.0 - dw) * p0.z + dw * p1.z};
    const double aMm = sqrt(dotd(aM, aM));
    const double ge = aE / (mass * (c * c));
    const double gq = aMm / mc;
    const double gp = sqrt(1.0 + gq * gq);
    if (!(gp < ge)) return;
    const double dp = mass * c * sqrt(ge * ge - gp * gp);
    V3d e2, e3;
    sk_basis(aM, aMm, e2, e3);
    const double eps = 6.283185307179586 * r.uniform();
    const double ce = cos(eps), se = sin(eps);
    const V3d ps = {aM.x + dp * (e2.x * ce + e3.x * se), aM.y + dp * (e2.y * ce + e3.y * se),
                    aM.z + dp * (e2.z * ce + e3.z * se)};
    const double gs0 = sqrt(dotd(ps, ps)) / mc;
    const double gs = sqrt(1.0 + gs0 * gs0);
    U = {ps.x / (mass * gs), ps.y / (mass * gs), ps.z / (mass * gs)};
}

// WeightCorrection by model for a pair of species weights wP, wQ: none,
// Nanbu (NanbuCorrection.C:50-66), SentokuKempNR, SentokuKemp.
__device__ void weight_correct_pair(int model, double wP, double wQ, double mP, double mQ, V3d preP, V3d preQ,
                                    V3d& UP, V3d& UQ, Rng& r) {
    if (model == 1) {
        const double u = r.uniform();
        if (u > wP / wQ) UQ = preQ;
        if (u > wQ / wP) UP = preP;
    } else if (model == 2 || model == 3) {
        const bool rel = model == 3;
        if (wP > wQ) {
            if (rel) sentoku_kemp(mP, wQ / wP, preP, UP, r);
            else sentoku_kemp_nr(mP, wQ / wP, preP, UP, r);
        } else if (wP < wQ) {
            if (rel) sentoku_kemp(mQ, wP / wQ, preQ, UQ, r);
            else sentoku_kemp_nr(mQ, wP / wQ, preQ, UQ, r);
        }
    }
}

// WeightCorrection (CoulombCollisionModel): none, Nanbu
// (NanbuCorrection.C:50-66), SentokuKempNR, SentokuKemp.
__device__ __forceinline__ void weight_correct(const CoulombSpecies& C, const CoulombParams& K, int a, int b,
                                               double wP, double wQ, V3d preP, V3d preQ, V3d& UP, V3d& UQ,
                                               Rng& r) {
    if (K.weight_corr == 1) {
        const double u = r.uniform();
        if (u > wP / wQ) UQ = preQ;
        if (u > wQ / wP) UP = preP;
    } else if (K.weight_corr == 2 || K.weight_corr == 3) {
        const bool rel = K.weight_corr == 3;
        if (wP > wQ) {
            if (rel) sentoku_kemp(C.m[a], wQ / wP, preP, UP, r);
            else sentoku_kemp_nr(C.m[a], wQ / wP, preP, UP, r);
        } else if (wP < wQ) {
            if (rel) sentoku_kemp(C.m[b], wP / wQ, preQ, UQ, r);
            else sentoku_kemp_nr(C.m[b], wP / wQ, preQ, UQ, r);
        }
    }
}

template <class R>
__device__ void nanbu_collide(const CoulombSpecies& C, const CoulombParams& K, int a, int ia, int b, int ib,
                              double lD, double nP, double nQ, double nPQ, Rng& r) {
    const double mP = C.m[a], qP = pcharge(C, a, ia), mQ = C.m[b], qQ = pcharge(C, b, ib);
    V3d UP = Vel<R>::get(C.p[a], ia), UQ = Vel<R>::get(C.p[b], ib);
    const double reMass = mP * mQ / (mP + mQ);
    const V3d g = {UP.x - UQ.x, UP.y - UQ.y, UP.z - UQ.z};
    const double gm = magd(g);
    double cl = K.cl;
    if (cl == 0.0) {
        double b0 = qP * qQ / (2.0 * kPi * eps0c() * reMass * gm * gm);
        if (K.calc_bmin) b0 = fmax(kPlanck / (2.0 * (gm * reMass)), fabs(b0));
        cl = fmax(2.0, 0.5 * log(1.0 + (lD * lD) / (b0 * b0)));
    }
    const double A = qP * qQ / (eps0c() * reMass);
    const double s = cl / (4.0 * kPi) * (A * A) * (nQ * nP / nPQ) * (1.0 / (gm * gm * gm)) * K.dt;
    const double cosChi = cos_chi(s, r);
    const double sinChi = sqrt(1.0 - cosChi * cosChi);
    const double gp = sqrt(g.y * g.y + g.z * g.z);
    const double eps = 2.0 * kPi * r.uniform();
    const double ce = cos(eps), se = sin(eps);
    const V3d h = {gp * ce, -1.0 * (g.y * g.x * ce + gm * g.z * se) / gp, -1.0 * (g.z * g.x * ce - gm * g.y * se) / gp};
    const V3d d = {(1.0 - cosChi) * g.x + sinChi * h.x, (1.0 - cosChi) * g.y + sinChi * h.y,
                   (1.0 - cosChi) * g.z + sinChi * h.z};
    const double kp = mQ / (mP + mQ), kq = mP / (mP + mQ);
    V3d nUP = {UP.x - kp * d.x, UP.y - kp * d.y, UP.z - kp * d.z};
    V3d nUQ = {UQ.x + kq * d.x, UQ.y + kq * d.y, UQ.z + kq * d.z};
    weight_correct(C, K, a, b, pweight(C, a, ia), pweight(C, b, ib), UP, UQ, nUP, nUQ, r);
    Vel<R>::put(C.p[a], ia, nUP);
    Vel<R>::put(C.p[b], ib, nUQ);
}

// PerezRelativisticCollision::collide (PerezRelativisticCollision.C:60-192),
// with the low-temperature cap s_max.
template <class R>
__device__ void perez_collide(const CoulombSpecies& C, const CoulombParams& K, int a, int ia, int b, int ib,
                              double lD, double nP, double nQ, double nPQ, Rng& r) {
    const double mP = C.m[a], qP = pcharge(C, a, ia), mQ = C.m[b], qQ = pcharge(C, b, ib);
    const V3d UP = Vel<R>::get(C.p[a], ia), UQ = Vel<R>::get(C.p[b], ib);
    CoM f;
    if (!com_frame(UP, UQ, mP, mQ, f)) return;
    const double mgsum = mP * f.gP + mQ * f.gQ;
    const double c2 = kC * kC;
    const double pc2 = f.mag_pc * f.mag_pc;
    const double e0 = eps0c();
    double cl = K.cl;
    if (cl == 0.0) {
        double b0 = qP * qQ / (4.0 * kPi * e0 * c2) * f.gc / mgsum * (1.0 + mP * f.gPc * mQ * f.gQc * c2 / pc2);
        if (K.calc_bmin) b0 = fmax(kPlanck / (2 * f.mag_pc), fabs(b0));
        cl = fmax(2.0, 0.5 * log(1.0 + (lD * lD) / (b0 * b0)));
    }
    const double t1 = f.gc * f.mag_pc / mgsum;
    const double t2b = 1.0 + mP * f.gPc * mQ * f.gQc * c2 / pc2;
    const double t2 = t2b * t2b;
    const double qq = qP * qQ;
    double s = (nP * nQ / nPQ) * K.dt * cl * (qq * qq) / (4.0 * kPi * (e0 * e0) * (c2 * c2) * mP * f.gP * mQ * f.gQ) *
               t1 * t2;
    const double v_rel = f.mag_pc * mgsum / (mP * f.gPc * mQ * f.gQc * f.gc);
    const double s_max = pow(4.0 * kPi / 3.0, 1.0 / 3.0) * (nP * nQ / nPQ) * K.dt * (mP + mQ) /
                         fmax(mP * pow(nP, 2.0 / 3.0), mQ * pow(nQ, 2.0 / 3.0)) * v_rel;
    s = fmin(s_max, s);
    const double cosChi = cos_chi(s, r);
    const double sinChi = sqrt(1.0 - cosChi * cosChi);
    const double eps = 2.0 * kPi * r.uniform();
    V3d nUP = UP, nUQ = UQ;
    com_rotate(f, cosChi, sinChi, eps, mP, mQ, nUP, nUQ);
    weight_correct(C, K, a, b, pweight(C, a, ia), pweight(C, b, ib), UP, UQ, nUP, nUQ, r);
    Vel<R>::put(C.p[a], ia, nUP);
    Vel<R>::put(C.p[b], ib, nUQ);
}

template <class R>
__device__ __forceinline__ void collide(const CoulombSpecies& C, const CoulombParams& K, int a, int ia, int b,
                                        int ib, double lD, double nP, double nQ, double nPQ, Rng& r) {
    if (K.perez) perez_collide<R>(C, K, a, ia, b, ib, lD, nP, nQ, nPQ, r);
    else nanbu_collide<R>(C, K, a, ia, b, ib, lD, nP, nQ, nPQ, r);
}

// CoulombCollisionModel::debyeLength (CoulombCollisionModel.C:249-309) over
// the colliding species of cell c, before any of its pairs collide, by the
// cell's warp: lane l sums the parcels l, l + 32, ... of a species, the
// lanes' sums are added in a fixed tree (lane l < off takes lane l + off's
// for off = 16 .. 1), so the result does not depend on scheduling.  Every
// lane returns the length.
__device__ __forceinline__ double warp_tree_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return __shfl_sync(0xffffffffu, v, 0);
}

template <class R>
__device__ double debye_length_warp(const CoulombSpecies& C, const CoulombParams& K, int c, int lane) {
    double debye = 0.0, n_max = 0.0;
    for (int k = 0; k < C.n; ++k) {
        double vSqr = 0.0, n = 0.0, charge = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
        const int s0 = C.start[k][c], s1 = C.start[k][c + 1];
        for (int t = s0 + lane; t < s1; t += 32) {
            const int i = C.idx[k][t];
            const V3d U = Vel<R>::get(C.p[k], i);
            const double w = pweight(C, k, i);
            vSqr += dotd(U, U) * w;
            charge += pcharge(C, k, i) * w;
            vx += w * U.x;
            vy += w * U.y;
            vz += w * U.z;
            n += w;
        }
        vSqr = warp_tree_sum(vSqr);
        charge = warp_tree_sum(charge);
        vx = warp_tree_sum(vx);
        vy = warp_tree_sum(vy);
        vz = warp_tree_sum(vz);
        n = warp_tree_sum(n);
        if (n <= 0.0) continue;
        V3d v = {vx / n, vy / n, vz / n};
        charge /= n;
        vSqr /= n;
        n /= K.vol[c];
        if (n > n_max) n_max = n;
        const double vd2 = K.debye_drift ? dotd(v, v) : 0.0;
        const double T = C.m[k] / (3.0 * kKb) * (vSqr - vd2);
        if (T <= 0.0) continue;
        debye += n * charge * charge / eps0c() * 1.0 / (T * kKb);
    }
    if (debye <= 0.0) return 0.0;
    const double r_min = pow(4.0 * kPi * n_max / 3.0, -1.0 / 3.0);
    return fmax(r_min, sqrt(1 / debye));
}

// ------------------------------------------------ Perez ionisation ---
// PerezIonizationModel (CoulombCollisionModel/IonizationModel/
// PerezIonizationModel/PerezIonizationModel.C:129-385) inside the Coulomb
// step: the pair densities of initIonization / prepareNumberDensities
// (lane 0, in the pairing order), prepareIonization before and ionize
// after each electron - ion collision.  The tables per species (C index):
// cross section, transferred and lost energy, each [Zstar][100].
struct PerezDev {
    int on;
    int ek;                                // C index of the electron species, -1: none
    int limit[PICGPU_MAX_SPECIES];         // ionisation limit per C index, -1: does not ionise
    int atomic[PICGPU_MAX_SPECIES];
    const double* tab[PICGPU_MAX_SPECIES];
    double mE;
    PerezElectron* out;
    unsigned long long* n_out;
    long cap;
};

// initIonization: np is the density of the pair's non-electron species
__device__ __forceinline__ void perez_init(const PerezDev& Z, int kp, int kq, double nP, double nQ, double& np,
                                           double& ne, double& nei) {
    ne = 0.0;
    nei = 0.0;
    if (kp == Z.ek) np = nQ;
    else if (kq == Z.ek) np = nP;
}

__device__ __forceinline__ double electron_eV(double mE, V3d U) {
    const double b = magd(U) / kC;
    const double gamma = 1.0 / sqrt(1.0 - b * b);
    return (gamma - 1.0) * mE * kC * kC / kEch;
}

__device__ __forceinline__ int zstar(const CoulombSpecies& C, int k, int i) {
    return C.p[k].zq ? C.p[k].zq[i] : 1;
}

// prepareNumberDensities for the pair (kp, ip), (kq, iq)
template <class R>
__device__ void perez_densities(const CoulombSpecies& C, const PerezDev& Z, int kp, int ip, int kq, int iq,
                                double& ne, double& nei) {
    int ke, ie, ki, ii;
    if (kp == Z.ek) { ke = kp; ie = ip; ki = kq; ii = iq; }
    else if (kq == Z.ek) { ke = kq; ie = iq; ki = kp; ii = ip; }
    else return;
    const int zs = zstar(C, ki, ii);
    if (Z.limit[ki] < 0 || zs >= Z.limit[ki]) return;
    double x = 6.142165 * log(electron_eV(Z.mE, Vel<R>::get(C.p[ke], ie)));
    if (x < 0.0) x = 0.0;
    else if (x > 99.0) x = 99.0;
    const double cs = Z.tab[ki][size_t(zs) * 100 + size_t(int(x))];
    if (cs > 0.0) {
        const double We = pweight(C, ke, ie), Wi = pweight(C, ki, ii);
        ne += We;
        nei += We < Wi ? We : Wi;
    }
}

// prepareIonization: 1 when (kp, ip) is the electron, 2 when (kq, iq) is,
// 0 when the pair does not ionise
__device__ __forceinline__ int perez_pair(const CoulombSpecies& C, const PerezDev& Z, int kp, int ip, int kq, int iq,
                                          double nei) {
    int which = 0, ki = 0, ii = 0;
    if (kp == Z.ek && Z.limit[kq] >= 0) { which = 1; ki = kq; ii = iq; }
    else if (kq == Z.ek && Z.limit[kp] >= 0) { which = 2; ki = kp; ii = ip; }
    if (!which || zstar(C, ki, ii) >= Z.limit[ki] || !(nei > 0.0)) return 0;
    return which;
}

// ionize for the electron (ke, ie) and the ion (ki, ii) after their
// collision; draws from the stream of the collision ordinal.  Returns 1 when
// the charge state rose.
template <class R>
__device__ int perez_ionize(const CoulombSpecies& C, const CoulombParams& K, const PerezDev& Z, int ke, int ie,
                            int ki, int ii, double np, double ne, double nei, uint32_t cell, uint32_t step,
                            long ord) {
    const int A = Z.atomic[ki];
    const double* cs = Z.tab[ki];
    const double* te = cs + size_t(A) * 100;
    const double* le = te + size_t(A) * 100;
    int Zstar = zstar(C, ki, ii);
    const int initialZstar = Zstar;
    const double c = kC;
    V3d Ue = Vel<R>::get(C.p[ke], ie);
    const V3d Ui = Vel<R>::get(C.p[ki], ii);
    const double me_ = magd(Ue), mi_ = magd(Ui);
    double gammaE = 1.0 / sqrt(1.0 - (me_ / c) * (me_ / c));
    const double gammaP = 1.0 / sqrt(1.0 - (mi_ / c) * (mi_ / c));
    const double massE = C.m[ke], massP = C.m[ki];
    const double wE = pweight(C, ke, ie), wP = pweight(C, ki, ii);
    const double wEwP = wE / wP;
    const double wPwE = 1.0 / wEwP;
    double gamma_s = gammaP * gammaE * (1.0 - mi_ * me_ / (c * c));
    if (gamma_s <= 1.0) return 0;
    Philox r(K.seed, kStreamIonize | uint32_t(ord), cell, step);
    const double ionCoeff_s = c * sqrt(gamma_s * gamma_s - 1.0) / gammaP * (np * ne / nei) * K.dt;
    const double eVkin_s = (gamma_s - 1.0) * massE * c * c / kEch;
    const double rndU = r.uniform();
    const int ionizationMax = Z.limit[ki] - Zstar - 1;
    double rate[PICGPU_PEREZ_MAX_Z], rate_inv[PICGPU_PEREZ_MAX_Z], prop[PICGPU_PEREZ_MAX_Z];
    double com = 0.0;
    int added = 0;
    for (int k = 0; k <= ionizationMax; ++k) {
        const double s = 6.142165 * log(eVkin_s);
        if (s < 0.0) break;
        const double* csz = cs + size_t(Zstar) * 100;
        const double* tez = te + size_t(Zstar) * 100;
        const double* lez = le + size_t(Zstar) * 100;
        double crossSection, transferred, lost;
        if (s < 99.0) {
            const int l = int(s);
            const double d = s - double(l);
            crossSection = (csz[l + 1] - csz[l]) * d + csz[l];
            transferred = (tez[l + 1] - tez[l]) * d + tez[l];
            lost = (lez[l + 1] - lez[l]) * d + lez[l];
        } else {
            const double d = s - 99.0;
            crossSection = (csz[99] - csz[98]) * d + csz[99];
            transferred = tez[99];
            lost = lez[99];
        }
        if (crossSection <= 0.0) break;
        if (lost > gamma_s - 1.0) break;
        rate[k] = ionCoeff_s * crossSection / gammaE;
        rate_inv[k] = 1.0 / rate[k];
        prop[k] = exp(-rate[k]);
        if (k == 0) {
            com = prop[k];
        } else {
            for (int x = 0; x < k; ++x) {
                double cp = 1.0 - rate[k] * rate_inv[x];
                for (int b = 0; b < x; ++b) cp *= 1.0 - rate[x] * rate_inv[b];
                for (int b = x + 1; b < k; ++b) cp *= 1.0 - rate[x] * rate_inv[b];
                if (k < ionizationMax) com += (prop[k] - prop[x]) / cp;
                else com += (1.0 - prop[k] + rate[k] * rate_inv[x] * (prop[x] - 1.0)) / cp;
            }
        }
        if (rndU < com) break;
        const V3d pOld = {Ue.x * gammaE * massE, Ue.y * gammaE * massE, Ue.z * gammaE * massE};
        const V3d pI = {Ui.x * gammaP * massP, Ui.y * gammaP * massP, Ui.z * gammaP * massP};
        const double p2 = gamma_s * gamma_s - 1.0;
        const double rndU2 = r.uniform();
        if (rndU2 < wEwP) {
            C.p[ki].zq[ii] += 1;
            const double gammaW = transferred + 1.0;
            const double alpha_w = sqrt((gammaW * gammaW - 1.0) / p2);
            const double f = gammaW - alpha_w * gamma_s;
            const V3d pNew = {alpha_w * pOld.x + f * pI.x * massE / massP, alpha_w * pOld.y + f * pI.y * massE / massP,
                              alpha_w * pOld.z + f * pI.z * massE / massP};
            const double gNew = sqrt(1.0 + pow(magd(pNew) / (massE * c), 2.0));
            const unsigned long long slot = atomicAdd(Z.n_out, 1ull);
            if (slot < (unsigned long long)Z.cap) {
                PerezElectron& o = Z.out[slot];
                o.key = (static_cast<unsigned long long>(cell) << 32) | (static_cast<unsigned long long>(ord) << 6) |
                        static_cast<unsigned long long>(k);
                o.tet = C.p[ke].tet[ie];
                for (int a = 0; a < 3; ++a) o.y[a] = sizeof(R) == 8 ? C.p[ke].y64[a][ie] : double(C.p[ke].y32[a][ie]);
                const double den = massE * gNew;
                o.U[0] = pNew.x / den;
                o.U[1] = pNew.y / den;
                o.U[2] = pNew.z / den;
                o.nw = wP;
            }
            ++added;
        }
        if (rndU2 < wPwE) {
            const double alpha_e = sqrt((pow(gamma_s - lost, 2.0) - 1.0) / p2);
            const double f = (1.0 - alpha_e) * gamma_s - lost;
            const V3d pLost = {alpha_e * pOld.x + f * pI.x * massE / massP, alpha_e * pOld.y + f * pI.y * massE / massP,
                               alpha_e * pOld.z + f * pI.z * massE / massP};
            const double gLost = sqrt(1.0 + pow(magd(pLost) / (massE * c), 2.0));
            const double den = massE * gLost;
            Ue = {pLost.x / den, pLost.y / den, pLost.z / den};
            Vel<R>::put(C.p[ke], ie, Ue);
            gammaE += ((1.0 - alpha_e) * gamma_s - lost) * gammaP;
            gamma_s -= lost;
        }
        Zstar++;
    }
    (void)added;
    return Zstar != initialZstar ? 1 : 0;
}

// One inter-species collision with prepareIonization before and ionize
// after it (which: perez_pair's answer for the pair as passed).
template <class R>
__device__ __forceinline__ int collide_ionize(const CoulombSpecies& C, const CoulombParams& K, const PerezDev& Z,
                                              int a, int ia, int b, int ib, double lD, double nP, double nQ,
                                              double nPQ, Rng& r, double np, double ne, double nei, uint32_t cell,
                                              uint32_t step, long ord) {
    const int which = Z.on ? perez_pair(C, Z, a, ia, b, ib, nei) : 0;
    collide<R>(C, K, a, ia, b, ib, lD, nP, nQ, nPQ, r);
    if (which == 1) return perez_ionize<R>(C, K, Z, a, ia, b, ib, np, ne, nei, cell, step, ord);
    if (which == 2) return perez_ionize<R>(C, K, Z, b, ib, a, ia, np, ne, nei, cell, step, ord);
    return 0;
}

// The random numbers of a cell's Coulomb step.  The shuffles take the
// uniforms of the cell's stream (seed, Coulomb, cell, step) in order: draw t
// is the (t & 1) half of counter block t / 2, so any lane can compute any
// draw.  The collision of ordinal k (its position in the sequential pairing
// order of the cell) draws from counter blocks 2^31 + 8 k on (at most three
// uniforms), so collisions of disjoint parcels can run on different lanes.
struct CellStream {
    uint64_t seed;
    uint32_t cell, step;
    __device__ double draw(long t) const {
        Philox p(seed, kStreamCoulomb, cell, step);
        p.c0 = uint32_t(t >> 1);
        p.block();
        p.used = int(t & 1) * 2;
        return p.uniform();
    }
    __device__ Rng collision(long k) const {
        Rng r(seed, kStreamCoulomb, cell, step);
        r.p.c0 = 0x80000000u + uint32_t(k) * 8u;
        return r;
    }
};

// Fisher-Yates over sel[0, n) with the draws nd, nd + 1, ... (draw
// nd + n - 1 - k picks the partner of position k): the lanes compute 32
// draws at a time, lane 0 applies their swaps in order.
__device__ void shuffle_warp(int* sel, int n, const CellStream& cs, long& nd, int lane) {
    for (int k = lane; k < n; k += 32) sel[k] = k;
    __syncwarp();
    for (int base = 0; base < n - 1; base += 32) {
        const int t = base + lane;
        int j = 0;
        if (t < n - 1) {
            const int k = n - 1 - t;
            j = int(cs.draw(nd + t) * double(k + 1));
            if (j > k) j = k;
        }
        const int m = min(32, n - 1 - base);
        for (int q = 0; q < m; ++q) {
            const int jq = __shfl_sync(0xffffffffu, j, q);
            if (lane == 0) {
                const int k = n - 1 - (base + q);
                const int tmp = sel[k];
                sel[k] = sel[jq];
                sel[jq] = tmp;
            }
        }
    }
    __syncwarp();
    nd += n > 1 ? n - 1 : 0;
}

// Per-warp shared buffers for the shuffled positions; larger cells use the
// species' global scratch (same layout as the cell lists).
constexpr int kCoulombWarps = 4;
constexpr int kCoulombShared = 512;

// NanbuYonemuraPairing::pairANDcollide (NanbuYonemuraPairing.C:56-325) and
// TakizukaAbePairing::pairANDcollide (TakizukaAbePairing.C:60-341), one warp
// per cell.  The pairings and their collision parameters are the sequential
// ones; each collision gets the random stream of its ordinal, and the lanes
// take chains of collisions that share no parcel: disjoint pairs one each,
// and where one parcel meets several partners (odd counts, unequal species
// counts) the partners of that parcel in their sequential order.
template <class R>
__global__ void __launch_bounds__(32 * kCoulombWarps) coulomb_kernel(CoulombSpecies C, CoulombParams K, PerezDev Z) {
    __shared__ int sh_sel[kCoulombWarps][2][kCoulombShared];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int c = int((long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
    if (c >= K.n_cells) return;  // warp-uniform
    const double V = K.vol[c];
    const CellStream cs{K.seed, uint32_t(c), K.step_dev ? *K.step_dev : K.step};
    const double lD = K.cl == 0.0 ? debye_length_warp<R>(C, K, c, lane) : 0.0;
    long nd = 0, ord = 0;
    unsigned long long pairs = 0, ionized = 0;
    const uint32_t step = cs.step;
    double np = 0.0, ne = 0.0, nei = 0.0;   // the ionisation model's pair densities
    for (int i = 0; i < C.n; ++i) {
        for (int jj = C.n - 1; jj >= i; --jj) {
            const int a = i, b = jj;
            const int sa = C.start[a][c], sb = C.start[b][c];
            const int nA = C.start[a][c + 1] - sa, nB = C.start[b][c + 1] - sb;
            const int* LA = C.idx[a] + sa;
            const int* LB = C.idx[b] + sb;
            // NanbuYonemuraPairing.C:96-113: the real particles of each
            // species, parcel by parcel in list order (lane 0)
            double sA = 0.0, sB = 0.0;
            if (!K.takizuka_abe) {
                if (lane == 0) {
                    for (int t = 0; t < nA; ++t) sA += pweight(C, a, LA[t]);
                    if (a != b)
                        for (int t = 0; t < nB; ++t) sB += pweight(C, b, LB[t]);
                }
                sA = __shfl_sync(0xffffffffu, sA, 0);
                sB = __shfl_sync(0xffffffffu, sB, 0);
            }
            if (a == b && nA > 1) {
                if (!K.allow_intra) continue;
                int* sel = nA <= kCoulombShared ? sh_sel[wib][0] : C.sel[a] + sa;
                shuffle_warp(sel, nA, cs, nd, lane);
                if (K.takizuka_abe) {
                    // TakizukaAbePairing.C:108-153: an odd count collides
                    // P-Q, Q-R and P-R (one chain), then pairs from the
                    // fourth parcel on
                    const double n = double(nA) * C.w[a] / V;
                    if (nA % 2 != 0) {
                        const double n12 = (double(nA) + 3.0) * C.w[a] / V;
                        if (lane == 0) {
                            const int P = LA[sel[0]], Q = LA[sel[1]], Rr = LA[sel[2]];
                            Rng r0 = cs.collision(ord), r1 = cs.collision(ord + 1), r2 = cs.collision(ord + 2);
                            collide<R>(C, K, a, P, a, Q, lD, n, n, n12, r0);
                            collide<R>(C, K, a, Q, a, Rr, lD, n, n, n12, r1);
                            collide<R>(C, K, a, P, a, Rr, lD, n, n, n12, r2);
                        }
                        const int np = (nA - 3) / 2;
                        for (int x = lane; x < np; x += 32) {
                            Rng r = cs.collision(ord + 3 + x);
                            collide<R>(C, K, a, LA[sel[3 + 2 * x]], a, LA[sel[4 + 2 * x]], lD, n, n, n12, r);
                        }
                        ord += 3 + np;
                        pairs += 2 + nA / 2;
                    } else {
                        const int np = nA / 2;
                        for (int x = lane; x < np; x += 32) {
                            Rng r = cs.collision(ord + x);
                            collide<R>(C, K, a, LA[sel[2 * x]], a, LA[sel[2 * x + 1]], lD, n, n, n, r);
                        }
                        ord += np;
                        pairs += nA / 2;
                    }
                    __syncwarp();
                    continue;
                }
                const double n = sA / V;
                if (nA % 2 != 0) {
                    // the pairs (0 1) (2 3) ... then (nA-1 0): the last
                    // collision follows the first one's on parcel sel[0]
                    // NanbuYonemuraPairing.C:128-141: real particles that
                    // collide, the extra pair first
                    double nAA = 0.0;
                    if (lane == 0) {
                        nAA += 2.0 * fmin(pweight(C, a, LA[sel[nA - 1]]), pweight(C, a, LA[sel[0]]));
                        for (int x = 0; x < nA - 2; x += 2)
                            nAA += 2.0 * fmin(pweight(C, a, LA[sel[x]]), pweight(C, a, LA[sel[x + 1]]));
                    }
                    const double n12 = __shfl_sync(0xffffffffu, nAA, 0) / V;
                    const int np = (nA - 1) / 2;
                    for (int x = lane; x < np; x += 32) {
                        Rng r = cs.collision(ord + x);
                        collide<R>(C, K, a, LA[sel[2 * x]], a, LA[sel[2 * x + 1]], lD, n, n, n12, r);
                        if (x == 0) {
                            Rng rl = cs.collision(ord + np);
                            collide<R>(C, K, a, LA[sel[nA - 1]], a, LA[sel[0]], lD, n, n, n12, rl);
                        }
                    }
                    ord += np + 1;
                    pairs += 1 + nA / 2;
                } else {
                    double nAA = 0.0;
                    if (lane == 0)
                        for (int x = 0; x < nA - 1; x += 2)
                            nAA += 2.0 * fmin(pweight(C, a, LA[sel[x]]), pweight(C, a, LA[sel[x + 1]]));
                    const double n12 = __shfl_sync(0xffffffffu, nAA, 0) / V;
                    const int np = nA / 2;
                    for (int x = lane; x < np; x += 32) {
                        Rng r = cs.collision(ord + x);
                        collide<R>(C, K, a, LA[sel[2 * x]], a, LA[sel[2 * x + 1]], lD, n, n, n12, r);
                    }
                    ord += np;
                    pairs += nA / 2;
                }
                __syncwarp();
            } else if (a != b && min(nA, nB) != 0) {
                if (nA == nB) {
                    int* sel = nA <= kCoulombShared ? sh_sel[wib][0] : C.sel[a] + sa;
                    shuffle_warp(sel, nA, cs, nd, lane);
                    double nP, nQ, nPQ;
                    if (K.takizuka_abe) {
                        nP = double(nA) * C.w[a] / V;
                        nQ = double(nB) * C.w[a] / V;
                        nPQ = nP;
                    } else {
                        nP = sA / V;
                        nQ = sB / V;
                        nPQ = 0.0;
                    }
                    // the pairs' real particles and the ionisation densities
                    // (initIonization, prepareNumberDensities), lane 0 in order
                    double nAB = 0.0;
                    if (lane == 0) {
                        if (Z.on) perez_init(Z, a, b, nP, nQ, np, ne, nei);
                        for (int k = 0; k < nA; ++k) {
                            if (!K.takizuka_abe)
                                nAB += fmin(pweight(C, a, LA[sel[k]]), pweight(C, b, LB[sel[nA - k - 1]]));
                            if (Z.on) perez_densities<R>(C, Z, a, LA[sel[k]], b, LB[sel[nA - k - 1]], ne, nei);
                        }
                    }
                    if (!K.takizuka_abe) nPQ = __shfl_sync(0xffffffffu, nAB, 0) / V;
                    np = __shfl_sync(0xffffffffu, np, 0);
                    ne = __shfl_sync(0xffffffffu, ne, 0);
                    nei = __shfl_sync(0xffffffffu, nei, 0);
                    for (int k = lane; k < nA; k += 32) {
                        Rng r = cs.collision(ord + k);
                        ionized += collide_ionize<R>(C, K, Z, a, LA[sel[k]], b, LB[sel[nA - k - 1]], lD, nP, nQ, nPQ,
                                                     r, np, ne, nei, uint32_t(c), step, ord + k);
                    }
                    ord += nA;
                    pairs += nA;
                } else {
                    const bool aMin = nA < nB;
                    const int minS = aMin ? a : b, maxS = aMin ? b : a;
                    const int* Lmin = aMin ? LA : LB;
                    const int* Lmax = aMin ? LB : LA;
                    const int nMax = max(nA, nB), nMin = min(nA, nB);
                    int* smin = nMin <= kCoulombShared ? sh_sel[wib][0] : C.sel[minS] + (aMin ? sa : sb);
                    int* smax = nMax <= kCoulombShared ? sh_sel[wib][1] : C.sel2[maxS] + (aMin ? sb : sa);
                    shuffle_warp(smin, nMin, cs, nd, lane);
                    shuffle_warp(smax, nMax, cs, nd, lane);
                    if (K.takizuka_abe) {
                        // TakizukaAbePairing.C:197-314: group 1 spreads the
                        // remainder nMax % nMin over delta + 1 partners each,
                        // group 2 gives the other minority parcels delta
                        // each; a lane takes one minority parcel's partners
                        const double nMinS = double(nMin) * C.w[a] / V, nMaxS = double(nMax) * C.w[a] / V;
                        const int delta = nMax / nMin;
                        const double delta_r = double(nMax % nMin) / double(nMin);
                        const int g1min = int(delta_r * double(nMin));
                        const int g1max = int(double(delta + 1) * delta_r * double(nMin));
                        const int g2min = int((1.0 - delta_r) * double(nMin));
                        const int g2max = int(double(delta) * (1.0 - delta_r) * double(nMin));
                        if (g1min > 0) {
                            if (Z.on) {
                                if (lane == 0) {
                                    perez_init(Z, minS, maxS, nMinS, nMaxS, np, ne, nei);
                                    for (int g = 0, q1 = 0; g < g1max; ++g, ++q1) {
                                        if (q1 >= g1min) q1 = 0;
                                        perez_densities<R>(C, Z, minS, Lmin[smin[q1]], maxS, Lmax[smax[g]], ne, nei);
                                    }
                                }
                                np = __shfl_sync(0xffffffffu, np, 0);
                                ne = __shfl_sync(0xffffffffu, ne, 0);
                                nei = __shfl_sync(0xffffffffu, nei, 0);
                            }
                            for (int k = lane; k < g1min && k < g1max; k += 32)
                                for (int g = k; g < g1max; g += g1min) {
                                    Rng r = cs.collision(ord + g);
                                    ionized += collide_ionize<R>(C, K, Z, maxS, Lmax[smax[g]], minS, Lmin[smin[k]], lD,
                                                                 nMaxS, nMinS, nMaxS, r, np, ne, nei, uint32_t(c), step,
                                                                 ord + g);
                                }
                            ord += g1max;
                            __syncwarp();
                        }
                        // minority position g1min + g mod g2min (all g1min
                        // when g2min is 0), majority g1max + g; the group's
                        // densities after group 1 collided
                        if (Z.on) {
                            if (lane == 0) {
                                perez_init(Z, minS, maxS, nMinS, nMaxS, np, ne, nei);
                                for (int g = 0, q1 = g1min; g < g2max; ++g, ++q1) {
                                    if (q1 >= g2min + g1min) q1 = g1min;
                                    perez_densities<R>(C, Z, minS, Lmin[smin[q1]], maxS, Lmax[smax[g1max + g]], ne, nei);
                                }
                            }
                            np = __shfl_sync(0xffffffffu, np, 0);
                            ne = __shfl_sync(0xffffffffu, ne, 0);
                            nei = __shfl_sync(0xffffffffu, nei, 0);
                        }
                        const int chains = g2min > 0 ? g2min : 1;
                        for (int k = lane; k < chains && k < g2max; k += 32)
                            for (int g = k; g < g2max; g += chains) {
                                Rng r = cs.collision(ord + g);
                                ionized += collide_ionize<R>(C, K, Z, maxS, Lmax[smax[g1max + g]], minS,
                                                             Lmin[smin[g1min + k]], lD, nMaxS, nMinS, nMaxS, r, np, ne,
                                                             nei, uint32_t(c), step, ord + g);
                            }
                        ord += g2max;
                        pairs += g1max + g2max;
                        __syncwarp();
                        continue;
                    }
                    const double nMaxS = (maxS == a ? sA : sB) / V;
                    const double nMinS = (maxS == a ? sB : sA) / V;
                    double nAB = 0.0;
                    if (lane == 0) {
                        if (Z.on) perez_init(Z, minS, maxS, nMinS, nMaxS, np, ne, nei);
                        for (int l = 0, k = 0; l < nMax; ++l, ++k) {
                            if (k >= nMin) k = 0;
                            nAB += fmin(pweight(C, minS, Lmin[smin[k]]), pweight(C, maxS, Lmax[smax[l]]));
                            if (Z.on) perez_densities<R>(C, Z, minS, Lmin[smin[k]], maxS, Lmax[smax[l]], ne, nei);
                        }
                    }
                    const double n12 = __shfl_sync(0xffffffffu, nAB, 0) / V;
                    np = __shfl_sync(0xffffffffu, np, 0);
                    ne = __shfl_sync(0xffffffffu, ne, 0);
                    nei = __shfl_sync(0xffffffffu, nei, 0);
                    // majority parcel l meets minority parcel l mod nMin
                    for (int k = lane; k < nMin; k += 32)
                        for (int l = k; l < nMax; l += nMin) {
                            Rng r = cs.collision(ord + l);
                            ionized += collide_ionize<R>(C, K, Z, maxS, Lmax[smax[l]], minS, Lmin[smin[k]], lD, nMaxS,
                                                         nMinS, n12, r, np, ne, nei, uint32_t(c), step, ord + l);
                        }
                    ord += nMax;
                    pairs += nMax;
                }
                __syncwarp();
            }
        }
    }
    if (pairs && lane == 0) atomicAdd(K.counts + 4, pairs);
    for (int off = 16; off > 0; off >>= 1) ionized += __shfl_down_sync(0xffffffffu, ionized, off);
    if (ionized && lane == 0) atomicAdd(K.counts + 20, ionized);
}

void launch_coulomb(const CoulombSpecies& C, const CoulombParams& K, const PerezDev& Z, bool mixed,
                    cudaStream_t stream) {
    const int threads = 32 * kCoulombWarps;
    const unsigned blocks = unsigned((long(K.n_cells) * 32 + threads - 1) / threads);
    if (mixed) coulomb_kernel<float><<<blocks, threads, 0, stream>>>(C, K, Z);
    else coulomb_kernel<double><<<blocks, threads, 0, stream>>>(C, K, Z);
}

// The electrons of this step's ionisations: sorted by their key (the order
// of picFoam's sequential loop) and appended to the electron store from slot
// first on, with their nParticle and charge modifier 1.
template <class R>
__global__ void perez_append_kernel(const PerezElectron* __restrict__ e, long n, DSpecies p, long first) {
    for (long j = blockIdx.x * long(blockDim.x) + threadIdx.x; j < n; j += long(gridDim.x) * blockDim.x) {
        const long d = first + j;
        p.tet[d] = e[j].tet;
        for (int a = 0; a < 3; ++a) {
            if (sizeof(R) == 8) {
                p.y64[a][d] = e[j].y[a];
                p.u64[a][d] = e[j].U[a];
            } else {
                p.y32[a][d] = float(e[j].y[a]);
                p.u32[a][d] = float(e[j].U[a]);
            }
        }
        p.nw[d] = e[j].nw;
        p.zq[d] = 1;
    }
}

template <class T>
cudaError_t dmalloc(T** p, size_t n) {
    return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T));
}

int grid_of(long n, int bs) { return int(std::max<long>(1, std::min<long>((n + bs - 1) / bs, 148L * 16))); }

}  // namespace

cudaError_t collide_set_tables(const TetConst& t) { return cudaMemcpyToSymbol(c_tetC, &t, sizeof t); }

namespace {

// Philox4x32-10 of the device generator, first uniform of stream (stream, cell, 0).
double host_uniform(uint64_t seed, uint32_t stream, uint32_t cell) {
    uint32_t key0 = uint32_t(seed), key1 = uint32_t(seed >> 32);
    uint32_t x0 = 0, x1 = stream, x2 = cell, x3 = 0;
    for (int rr = 0; rr < 10; ++rr) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * x0, p1 = uint64_t(0xCD9E8D57u) * x2;
        const uint32_t n0 = uint32_t(p1 >> 32) ^ x1 ^ key0, n2 = uint32_t(p0 >> 32) ^ x3 ^ key1;
        x1 = uint32_t(p1); x3 = uint32_t(p0); x0 = n0; x2 = n2;
        key0 += 0x9E3779B9u; key1 += 0xBB67AE85u;
    }
    const uint32_t a = x0 >> 5, b = x1 >> 6;
    return (double(a) * 67108864.0 + double(b)) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------- binary (neutral) collisions --
// BinaryCollisionModel::performCollisions (BinaryCollisionModel.C:229-373)
// and performBackgroundCollisions (:375-515) with IsotropicScattering
// (IsotropicScattering.C:67-139), one thread per cell, candidates in the
// reference's order from the cell's own Philox streams.
struct BinaryParams {
    int n_cells;
    const double* vol;
    const int* cell_class;
    const double* offset;             // 24 per geometry class
    int ns;                           // neutral species
    double m[PICGPU_MAX_SPECIES], w[PICGPU_MAX_SPECIES], d[PICGPU_MAX_SPECIES], om[PICGPU_MAX_SPECIES];
    double G[PICGPU_MAX_SPECIES][PICGPU_MAX_SPECIES];   // exp(lgamma(2.5 - omega_PQ)) (VHS)
    const int* start[PICGPU_MAX_SPECIES];
    const int* idx[PICGPU_MAX_SPECIES];
    DSpecies p[PICGPU_MAX_SPECIES];
    int vhs, weight_corr;
    double tref;
    double* smax;
    double* rem;
    double* bgrem;
    int* list;
    int* oct;
    double dt;
    uint64_t seed;
    uint32_t step;
    const unsigned* step_dev;
    // background gas (uniformBackground)
    int bg;
    double bg_n, bg_T, bg_m, bg_d, bg_om, bg_u[3];
    double Gbg[PICGPU_MAX_SPECIES];
    unsigned long long* counts;
};

// TotalCrossSectionModel::sigmaTcR: HardSphere (HardSphere.C:47-70) or
// VariableHardSphere (VariableHardSphere.C:48-85).
__device__ double sigma_tcr(const BinaryParams& B, double dP, double dQ, double omP, double omQ, double mP,
                            double mQ, double G, V3d UP, V3d UQ) {
    const double dPQ = 0.5 * (dP + dQ);
    const V3d g = {UP.x - UQ.x, UP.y - UQ.y, UP.z - UQ.z};
    const double cR = sqrt(dotd(g, g));
    if (cR < 1.0e-300) return 0.0;
    double sig;
    if (B.vhs) {
        const double omPQ = 0.5 * (omP + omQ);
        const double mR = mP * mQ / (mP + mQ);
        sig = kPi * dPQ * dPQ * pow(2.0 * kKb * B.tref / (mR * cR * cR), omPQ - 0.5) / G;
    } else {
        sig = kPi * dPQ * dPQ;
    }
    return sig * cR;
}

// IsotropicScattering::updateVelocity: isotropic post-collision relative
// velocity in the centre-of-mass frame.
__device__ void iso_scatter(double mP, double mQ, V3d& UP, V3d& UQ, Rng& r) {
    const double M = mP + mQ;
    const V3d Ucm = {(mP * UP.x + mQ * UQ.x) / M, (mP * UP.y + mQ * UQ.y) / M, (mP * UP.z + mQ * UQ.z) / M};
    const V3d g = {UP.x - UQ.x, UP.y - UQ.y, UP.z - UQ.z};
    const double cR = sqrt(dotd(g, g));
    const double cosT = 2.0 * r.uniform() - 1.0;
    const double sinT = sqrt(1.0 - cosT * cosT);
    const double phi = 6.283185307179586 * r.uniform();
    const V3d pr = {cR * cosT, cR * (sinT * cos(phi)), cR * (sinT * sin(phi))};
    UP = {Ucm.x + pr.x * mQ / M, Ucm.y + pr.y * mQ / M, Ucm.z + pr.z * mQ / M};
    UQ = {Ucm.x - pr.x * mP / M, Ucm.y - pr.y * mP / M, Ucm.z - pr.z * mP / M};
}

// The cell-relative position of particle i of species k: y1 a + y2 b + y3 c
// with the corner offsets of its tet's face triangle.
template <class R>
__device__ int octant(const BinaryParams& B, int k, int i) {
    const int tet = B.p[k].tet[i];
    const int cell = tet / 12, t = tet - 12 * cell;
    const double* off = B.offset + size_t(B.cell_class[cell]) * 24;
    double y[3];
    if (sizeof(R) == 8) {
        y[0] = B.p[k].y64[0][i]; y[1] = B.p[k].y64[1][i]; y[2] = B.p[k].y64[2][i];
    } else {
        y[0] = B.p[k].y32[0][i]; y[1] = B.p[k].y32[1][i]; y[2] = B.p[k].y32[2][i];
    }
    double rel[3];
    for (int a = 0; a < 3; ++a)
        rel[a] = y[0] * off[3 * c_tetC.tri[t][0] + a] + y[1] * off[3 * c_tetC.tri[t][1] + a] +
                 y[2] * off[3 * c_tetC.tri[t][2] + a];
    // pos0(x) + 2 pos0(y) + 4 pos0(z)
    return (rel[0] >= 0.0 ? 1 : 0) + (rel[1] >= 0.0 ? 2 : 0) + (rel[2] >= 0.0 ? 4 : 0);
}

template <class R>
__global__ void __launch_bounds__(64) binary_kernel(BinaryParams B) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= B.n_cells) return;
    const uint32_t step = B.step_dev ? *B.step_dev : B.step;
    int cnt[PICGPU_MAX_SPECIES], off[PICGPU_MAX_SPECIES];
    int nC = 0, base = 0;
    double wmax = 0.0;
    for (int k = 0; k < B.ns; ++k) {
        const int s0 = B.start[k][c];
        cnt[k] = B.start[k][c + 1] - s0;
        off[k] = nC;
        nC += cnt[k];
        base += s0;
        if (cnt[k] > 0 && B.w[k] > wmax) wmax = B.w[k];
    }
    auto locate = [&](int j, int& k, int& i) {
        k = 0;
        while (k + 1 < B.ns && off[k + 1] <= j) ++k;
        i = B.idx[k][B.start[k][c] + (j - off[k])];
    };
    unsigned long long tested = 0, collided = 0, btested = 0, bcollided = 0;
    if (nC > 1) {
        int* L = B.list + base;
        int* O = B.oct + base;
        int scount[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = 0; j < nC; ++j) {
            int k, i;
            locate(j, k, i);
            const int o = octant<R>(B, k, i);
            O[j] = o;
            ++scount[o];
        }
        int soff[8], cur[8];
        int acc = 0;
        for (int o = 0; o < 8; ++o) {
            soff[o] = acc;
            cur[o] = acc;
            acc += scount[o];
        }
        for (int j = 0; j < nC; ++j) L[cur[O[j]]++] = j;
        const double smax0 = B.smax[c];
        const double sel = B.rem[c] + 0.5 * double(nC) * double(nC - 1) * wmax * smax0 * B.dt / B.vol[c];
        const long long nCand = (long long)sel;
        B.rem[c] = sel - double(nCand);
        Rng r(B.seed, kStreamBinary, uint32_t(c), step);
        for (long long q = 0; q < nCand; ++q) {
            const int P = int(r.uniform() * double(nC));
            const int oP = O[P];
            const int nSC = scount[oP];
            int Q = P;
            for (int it = 0; it < 1000 && Q == P; ++it) {
                if (nSC > 1) Q = L[soff[oP] + int(r.uniform() * double(nSC))];
                else Q = int(r.uniform() * double(nC));
            }
            if (Q == P) continue;
            int kP, iP, kQ, iQ;
            locate(P, kP, iP);
            locate(Q, kQ, iQ);
            V3d UP = Vel<R>::get(B.p[kP], iP), UQ = Vel<R>::get(B.p[kQ], iQ);
            const double sTcR =
                sigma_tcr(B, B.d[kP], B.d[kQ], B.om[kP], B.om[kQ], B.m[kP], B.m[kQ], B.G[kP][kQ], UP, UQ);
            ++tested;
            if (sTcR > B.smax[c]) B.smax[c] = sTcR;
            if (sTcR / smax0 > r.uniform()) {
                const V3d preP = UP, preQ = UQ;
                iso_scatter(B.m[kP], B.m[kQ], UP, UQ, r);
                weight_correct_pair(B.weight_corr, B.w[kP], B.w[kQ], B.m[kP], B.m[kQ], preP, preQ, UP, UQ, r);
                Vel<R>::put(B.p[kP], iP, UP);
                Vel<R>::put(B.p[kQ], iQ, UQ);
                ++collided;
            }
        }
    }
    if (B.bg && nC > 0) {
        const double smaxb = B.smax[c];
        const double coll = B.bgrem[c] + double(nC) * B.bg_n * smaxb * B.dt;
        const long long nCand = (long long)coll;
        B.bgrem[c] = coll - double(nCand);
        Rng r(B.seed, kStreamBinaryBg, uint32_t(c), step);
        const double vth = sqrt(kKb * B.bg_T / B.bg_m);
        for (long long q = 0; q < nCand; ++q) {
            const int P = int(r.uniform() * double(nC));
            int k, i;
            locate(P, k, i);
            V3d UP = Vel<R>::get(B.p[k], i);
            const double n0 = r.normal(), n1 = r.normal(), n2 = r.normal();
            V3d Ub = {vth * n0 + B.bg_u[0], vth * n1 + B.bg_u[1], vth * n2 + B.bg_u[2]};
            const double sTcR = sigma_tcr(B, B.d[k], B.bg_d, B.om[k], B.bg_om, B.m[k], B.bg_m, B.Gbg[k], UP, Ub);
            ++btested;
            if (sTcR > B.smax[c]) B.smax[c] = sTcR;
            if (sTcR / smaxb > r.uniform()) {
                iso_scatter(B.m[k], B.bg_m, UP, Ub, r);
                Vel<R>::put(B.p[k], i, UP);
                ++bcollided;
            }
        }
    }
    if (tested) atomicAdd(B.counts + 8, tested);
    if (collided) atomicAdd(B.counts + 9, collided);
    if (btested) atomicAdd(B.counts + 10, btested);
    if (bcollided) atomicAdd(B.counts + 11, bcollided);
}

// Table k of a packed cross-section block (energies first), linear between
// the bracketing nodes (ListCrossSection.C:33-88).
double host_xs(const std::vector<double>& xs, int n, int k, double x) {
    const double* e = xs.data();
    const double* v = xs.data() + size_t(k) * n;
    if (x <= e[0]) return v[0];
    if (x >= e[n - 1]) return v[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (e[mid] <= x) lo = mid; else hi = mid;
    }
    if (e[lo] == x) return v[lo];
    return v[lo] + ((x - e[lo]) / (e[hi] - e[lo])) * (v[hi] - v[lo]);
}

// FindMaximum (sigma v)_max over [0, emax) of the summed tables 1..n_tables-1
// (ElectronNeutralCollisionModel.C:383-424, IonNeutralCollisionModel.C:284-333).
double find_maximum(const std::vector<double>& xs, int n, int n_tables, double mass, double emax, double step) {
    if (!(emax > 0)) emax = xs[n - 1];
    if (!(step > 0)) step = emax / 100000.0;
    double sv = 0.0;
    for (double eV = 0.0; eV < emax; eV += step) {
        double q = 0.0;
        for (int k = 1; k < n_tables; ++k) q += host_xs(xs, n, k, eV);
        sv = std::fmax(sv, std::sqrt(2.0 * kEch * eV / mass) * q);
    }
    return sv;
}

// Uploads (sigma v)_max, remainders seeded U(0,1) from one Philox stream per
// cell, and the packed tables.
int upload_mcc(double** svmax, double** rem, double** xs_d, const std::vector<double>& xs, double sv,
               uint64_t seed, uint32_t stream, int nc, cudaStream_t s, std::string* msg) {
    std::vector<double> svm(nc, sv), r(nc);
    for (int c = 0; c < nc; ++c) r[c] = host_uniform(seed, stream, uint32_t(c));
    if (dmalloc(svmax, nc) || dmalloc(rem, nc) || dmalloc(xs_d, xs.size())) {
        *msg = "MCC state: device allocation failed";
        return PICGPU_OOM;
    }
    cudaMemcpyAsync(*svmax, svm.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(*rem, r.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(*xs_d, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "MCC state: upload failed";
        return PICGPU_CUDA_ERROR;
    }
    return PICGPU_OK;
}

bool ascending(const double* e, int n) {
    for (int i = 1; i < n; ++i)
        if (!(e[i] > e[i - 1])) return false;
    return true;
}

}  // namespace

namespace {

// IonizationData::calculateIonizationCrossSection (PerezIonizationModel.C:
// 405-484): per charge state Z the cross section summed over the orbitals
// k (Carlson binding energies, bindingEnergy :395-399; orbitals of equal
// binding energy counted together) and the energies transferred to the new
// electron and lost by the colliding one, averaged over the orbitals (units
// of m_e c^2), on 100 energies log-spaced over 1 eV - 10 MeV.  Layout:
// cs[Z][100], then transferred, then lost.
std::vector<double> perez_tables(const picgpu_perez_ion& in) {
    const int A = in.atomic_number;
    std::vector<double> t(size_t(3) * A * 100, 0.0);
    double* cs = t.data();
    double* te = cs + size_t(A) * 100;
    double* le = te + size_t(A) * 100;
    const double r_e = 2.8179403227e-15;
    const double step = 99.0 / std::log(1e7 / 1.0);
    auto bind = [&](int Z, int k) { return in.ionization_energy[Z] - in.binding_energy[A - Z - 1] + in.binding_energy[k]; };
    for (int Z = 0; Z < A; ++Z)
        for (int i = 0; i < 100; ++i) {
            const double E = std::exp(double(i) / step);
            int N = 1;
            double sig = 0.0, tr = 0.0, lo = 0.0;
            for (int k = 0; k < A - Z; ++k) {
                const double Bk = bind(Z, k);
                if (k < A - Z - 1 && Bk == bind(Z, k + 1)) {
                    N++;
                    continue;
                }
                const double eps = E / Bk;
                if (eps > 1.0) {
                    const double b_dash = Bk / 510997.37, eps_dash = E / 510997.37, u_dash = b_dash;
                    const double beta_eps2 = 1.0 - 1.0 / ((1.0 + eps_dash) * (1.0 + eps_dash));
                    const double beta_b2 = 1.0 - 1.0 / ((1.0 + b_dash) * (1.0 + b_dash));
                    const double beta_u2 = 1.0 - 1.0 / ((1.0 + u_dash) * (1.0 + u_dash));
                    const double sigma0 = 2.0 * kPi * r_e * r_e * N / (b_dash * (beta_eps2 + beta_b2 + beta_u2));
                    double ediv2 = 1.0 + eps_dash * 0.5;
                    ediv2 *= ediv2;
                    const double A1 = 1.0 / (1.0 + eps) * (1.0 + 2 * eps_dash) / ediv2;
                    const double A2 = (eps - 1.0) / 2.0 * b_dash * b_dash / ediv2;
                    const double A3 = std::log(beta_eps2 / (1.0 - beta_eps2)) - beta_eps2 - std::log(2.0 * b_dash);
                    const double sk = sigma0 * (0.5 * A3 * (1.0 - 1.0 / (eps * eps)) + 1.0 - 1.0 / eps + A2 -
                                                A1 * std::log(eps));
                    const double wk = sigma0 * (0.5 * A3 * (eps - 1.0) * (eps - 1.0) / (eps * (eps - 1.0)) +
                                                2.0 * std::log((eps + 1.0) * 0.5) - std::log(eps) +
                                                A2 * (eps - 1.0) * 0.25 -
                                                A1 * (std::log(eps) - (eps + 1.0) * std::log(0.5 * (eps + 1.0))));
                    sig += sk;
                    tr += wk * b_dash;
                    lo += (sk + wk) * b_dash;
                }
                N = 1;
            }
            if (sig > 0.0) {
                tr /= sig;
                lo /= sig;
            }
            cs[size_t(Z) * 100 + i] = sig;
            te[size_t(Z) * 100 + i] = tr;
            le[size_t(Z) * 100 + i] = lo;
        }
    return t;
}

}  // namespace

int collide_init(CollideState& st, const picgpu_config& cfg, const DMesh& m, cudaStream_t s, std::string* msg) {
    st.enabled = cfg.mcc.enabled || cfg.coulomb.enabled || cfg.ion_mcc.enabled || cfg.binary.enabled ||
                 cfg.merging.enabled;
    if (!st.enabled) return PICGPU_OK;
    const int nc = m.n_cells;
    if (dmalloc(&st.cell_start, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) ||
        dmalloc(&st.cell_count, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) || dmalloc(&st.cell_cursor, nc + 1) ||
        dmalloc(&st.counts, kCollideCounts) || dmalloc(&st.scan_tmp, (nc + 1) / 1024 + 8) || dmalloc(&st.overflow, 1) ||
        (cfg.mcc.enabled && dmalloc(&st.iz_cell, nc))) {
        *msg = "collision state: device allocation failed";
        return PICGPU_OOM;
    }
    cudaMemsetAsync(st.overflow, 0, sizeof(int), s);
    cudaMemsetAsync(st.counts, 0, kCollideCounts * sizeof(unsigned long long), s);
    if (st.iz_cell) cudaMemsetAsync(st.iz_cell, 0, size_t(nc) * sizeof(unsigned long long), s);
    if (cfg.perez.enabled) {
        // PerezIonizationModel.C:30-118: one entry per ion species; a limit
        // below 1 switches the species off
        const picgpu_perez& pz = cfg.perez;
        const int es = cfg.electron_species;
        bool ok = cfg.coulomb.enabled && es >= 0 && es < cfg.n_species && cfg.species[es].charge != 0.0 &&
                  pz.n_ions >= 0 && pz.n_ions <= PICGPU_PEREZ_MAX_IONS;
        for (int k = 0; ok && k < pz.n_ions; ++k) {
            const picgpu_perez_ion& in = pz.ion[k];
            ok = in.species >= 0 && in.species < cfg.n_species && in.species != es && in.atomic_number >= 1 &&
                 in.atomic_number <= PICGPU_PEREZ_MAX_Z;
            if (!ok || in.ionization_limit == 0) continue;
            const std::vector<double> t = perez_tables(in);
            if (dmalloc(&st.ptab[in.species], t.size()) ||
                cudaMemcpy(st.ptab[in.species], t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice) !=
                    cudaSuccess) {
                *msg = "Perez ionisation: device allocation failed";
                return PICGPU_OOM;
            }
            st.patomic[in.species] = in.atomic_number;
            st.plimit[in.species] = in.ionization_limit < 0 ? in.atomic_number
                                                            : std::min(in.ionization_limit, in.atomic_number);
        }
        if (!ok) {
            *msg = "Perez ionisation: bad settings (needs Coulomb collisions, a charged electron species and "
                   "ion species other than it, atomic numbers 1 - 64)";
            return PICGPU_INVALID_ARG;
        }
        st.pstage_cap = 1 << 20;
        if (dmalloc(&st.pstage, st.pstage_cap) || dmalloc(&st.pcount, 1)) {
            *msg = "Perez ionisation: device allocation failed";
            return PICGPU_OOM;
        }
    }
    if (cfg.merging.enabled) {
        // PairMerging.C:35-68: the settings and the species list
        const picgpu_merging& mg = cfg.merging;
        if (mg.n_species < 1 || mg.n_species > PICGPU_MAX_SPECIES || mg.n_check_neighbors < 1 ||
            !(mg.reduction_factor > 0.0 && mg.reduction_factor <= 1.0) || mg.cell_parcels_max < 1 ||
            mg.max_checks < 0 || mg.merge_maximum_per_cell < 0 || !(mg.velocity_ratio >= 0.0)) {
            *msg = "PairMerging: bad settings";
            return PICGPU_INVALID_ARG;
        }
        if (double(mg.cell_parcels_max) * mg.reduction_factor < double(mg.n_check_neighbors)) {
            *msg = "PairMerging: cellParcelsMax x reductionFactor is below nCheckNeighbors";
            return PICGPU_INVALID_ARG;
        }
        for (int k = 0; k < mg.n_species; ++k)
            if (mg.species[k] < 0 || mg.species[k] >= cfg.n_species) {
                *msg = "PairMerging: species not defined";
                return PICGPU_INVALID_ARG;
            }
    }
    if (cfg.coulomb.enabled) {
        const picgpu_coulomb& co = cfg.coulomb;
        if (co.pairing < 0 || co.pairing > 1 || co.collide < 0 || co.collide > 1 || co.coulomb_log < 0 ||
            co.weight_correction < 0 || co.weight_correction > 3) {
            *msg = "Coulomb: unknown pairing, collide or weight-correction model";
            return PICGPU_INVALID_ARG;
        }
        if (co.pairing == 1) {
            // TakizukaAbePairing.C:45-46: equal parcel weights only
            double w = -1.0;
            for (int k = 0; k < cfg.n_species; ++k) {
                if (cfg.species[k].charge == 0.0 || !cfg.species[k].solve_movement) continue;
                if (w < 0) w = cfg.species[k].weight;
                else if (cfg.species[k].weight != w) {
                    *msg = "Coulomb: TakizukaAbe pairing needs equal species weights";
                    return PICGPU_INVALID_ARG;
                }
            }
        }
    }
    if (cfg.mcc.enabled) {
        const picgpu_mcc& mc = cfg.mcc;
        if (mc.n_xs < 2 || mc.n_xs > PICGPU_MAX_XS_POINTS || !mc.xs_energy || !mc.xs_elastic || !mc.xs_excitation ||
            !mc.xs_ionization) {
            *msg = "MCC: cross-section tables missing";
            return PICGPU_INVALID_ARG;
        }
        if (cfg.electron_species < 0 || cfg.electron_species >= cfg.n_species) {
            *msg = "MCC: electron species not set";
            return PICGPU_INVALID_ARG;
        }
        if (mc.create_ion && (mc.ion_species < 0 || mc.ion_species >= cfg.n_species)) {
            *msg = "MCC: createIon needs an ion species";
            return PICGPU_INVALID_ARG;
        }
        if (!ascending(mc.xs_energy, mc.n_xs)) {
            *msg = "MCC: cross-section energies must ascend";
            return PICGPU_INVALID_ARG;
        }
        // the parcel weights of the store are per species: secondaries carry the
        // background weight, so it must equal the species weights
        if (mc.gas_weight != cfg.species[cfg.electron_species].weight ||
            (mc.create_ion && mc.gas_weight != cfg.species[mc.ion_species].weight)) {
            *msg = "MCC: background nEquivalentParticles must equal the electron and ion weights";
            return PICGPU_NOT_SUPPORTED;
        }
        st.n_xs = mc.n_xs;
        std::vector<double> xs(4 * size_t(mc.n_xs));
        for (int i = 0; i < mc.n_xs; ++i) {
            xs[i] = mc.xs_energy[i];
            xs[mc.n_xs + i] = mc.xs_elastic[i];
            xs[2 * mc.n_xs + i] = mc.xs_excitation[i];
            xs[3 * mc.n_xs + i] = mc.xs_ionization[i];
        }
        double sv = mc.sigma_v_max_init;
        if (!(sv > 0))
            sv = find_maximum(xs, mc.n_xs, 4, cfg.species[cfg.electron_species].mass, mc.find_max_energy,
                              mc.find_energy_step);
        st.svmax_init = sv;
        // remainders seeded U(0,1) (ElectronNeutralCollisionModel.C:286-296)
        const int e = upload_mcc(&st.svmax, &st.remainder, &st.xs, xs, sv, cfg.seed, kStreamRemainder, nc, s, msg);
        if (e) return e;
        // the FP32 copy the FP32 store's MCC kernel reads
        const std::vector<float> xs32(xs.begin(), xs.end());
        if (dmalloc(&st.xs32, xs32.size()) ||
            cudaMemcpy(st.xs32, xs32.data(), xs32.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
            *msg = "MCC tables: device allocation failed";
            return PICGPU_OOM;
        }
        if (dmalloc(&st.ncand, nc + 1) || dmalloc(&st.cand_off, nc + 2)) {
            *msg = "MCC state: device allocation failed";
            return PICGPU_OOM;
        }
        if (mc.neutral_parcels) {
            const int ns = mc.neutral_species;
            if (ns < 0 || ns >= cfg.n_species || cfg.species[ns].charge != 0.0) {
                *msg = "MCC: neutral_species must name a species of charge 0";
                return PICGPU_INVALID_ARG;
            }
            const double wn = cfg.species[ns].weight;
            if (wn != cfg.species[cfg.electron_species].weight ||
                (mc.create_ion && wn != cfg.species[mc.ion_species].weight)) {
                *msg = "MCC: neutral parcels need the electron and ion weights of the neutral species";
                return PICGPU_NOT_SUPPORTED;
            }
            if (cfg.binary.enabled) {
                *msg = "MCC: neutral-parcel collisions together with BinaryCollisionModel are not supported";
                return PICGPU_NOT_SUPPORTED;
            }
            // the same start value; remainders from their own stream
            double* xs_unused = nullptr;
            const int e2 = upload_mcc(&st.psvmax, &st.premainder, &xs_unused, xs, sv, cfg.seed, kStreamRemainder | 1u,
                                      nc, s, msg);
            if (e2) return e2;
            cudaFree(xs_unused);
            if (dmalloc(&st.n_live, nc)) {
                *msg = "MCC: device allocation failed";
                return PICGPU_OOM;
            }
        }
    }
    if (cfg.ion_mcc.enabled) {
        const picgpu_ion_mcc& im = cfg.ion_mcc;
        if (im.n_xs < 2 || im.n_xs > PICGPU_MAX_XS_POINTS || !im.xs_energy || !im.xs_elastic ||
            !im.xs_charge_exchange) {
            *msg = "ion MCC: cross-section tables missing";
            return PICGPU_INVALID_ARG;
        }
        if (im.ion_species < 0 || im.ion_species >= cfg.n_species) {
            *msg = "ion MCC: ion species not set";
            return PICGPU_INVALID_ARG;
        }
        if ((!(cfg.mcc.gas_density > 0) && !im.neutral_parcels) || !(cfg.mcc.gas_mass > 0)) {
            *msg = "ion MCC: background gas (mcc.gas_*) not set";
            return PICGPU_INVALID_ARG;
        }
        if (!ascending(im.xs_energy, im.n_xs)) {
            *msg = "ion MCC: cross-section energies must ascend";
            return PICGPU_INVALID_ARG;
        }
        st.n_ixs = im.n_xs;
        std::vector<double> xs(3 * size_t(im.n_xs));
        for (int i = 0; i < im.n_xs; ++i) {
            xs[i] = im.xs_energy[i];
            xs[im.n_xs + i] = im.xs_elastic[i];
            xs[2 * im.n_xs + i] = im.xs_charge_exchange[i];
        }
        double sv = im.sigma_v_max_init;
        if (!(sv > 0))
            sv = find_maximum(xs, im.n_xs, 3, cfg.species[im.ion_species].mass, im.find_max_energy,
                              im.find_energy_step);
        // remainders seeded U(0,1) (IonNeutralCollisionModel.C:199)
        const int e =
            upload_mcc(&st.isvmax, &st.iremainder, &st.ixs, xs, sv, cfg.seed, kStreamIonRemainder, nc, s, msg);
        if (e) return e;
        if (im.neutral_parcels) {
            const int ns = im.neutral_species;
            if (ns < 0 || ns >= cfg.n_species || cfg.species[ns].charge != 0.0 || cfg.binary.enabled) {
                *msg = "ion MCC: neutral_species must name a species of charge 0 (and no BinaryCollisionModel)";
                return PICGPU_INVALID_ARG;
            }
            if (im.weight_correction < PICGPU_WEIGHT_CORRECTION_NONE ||
                im.weight_correction > PICGPU_WEIGHT_CORRECTION_SENTOKU_KEMP) {
                *msg = "ion MCC: unknown weight-correction model";
                return PICGPU_INVALID_ARG;
            }
            double* xs_unused = nullptr;
            const int e2 = upload_mcc(&st.ipsvmax, &st.ipremainder, &xs_unused, xs, sv, cfg.seed,
                                      kStreamIonRemainder | 1u, nc, s, msg);
            if (e2) return e2;
            cudaFree(xs_unused);
        }
    }
    if (cfg.binary.enabled) {
        const picgpu_binary& bc = cfg.binary;
        if (bc.cross_section < 0 || bc.cross_section > 1 || bc.weight_correction < 0 || bc.weight_correction > 3 ||
            bc.background_species >= cfg.n_species) {
            *msg = "binary collisions: unknown cross-section or weight-correction model";
            return PICGPU_INVALID_ARG;
        }
        int first = -1;
        for (int k = 0; k < cfg.n_species; ++k) {
            if (cfg.species[k].charge != 0.0) continue;
            if (first < 0) first = k;
            if (!(bc.diameter[k] > 0)) {
                *msg = "binary collisions: every neutral species needs a diameter";
                return PICGPU_INVALID_ARG;
            }
        }
        if (bc.cross_section == PICGPU_XS_VARIABLE_HARD_SPHERE && !(bc.tref > 0)) {
            *msg = "binary collisions: VariableHardSphere needs Tref";
            return PICGPU_INVALID_ARG;
        }
        // picSigmaTcRMax: given, or BinaryCollisionModel::initialize
        // (BinaryCollisionModel.C:548-600): sigmaT v_mp(T) of the background
        // species when set, else of the first neutral species
        double smax = bc.sigma_tcr_max_init;
        if (!(smax > 0)) {
            const int sp = bc.background_species >= 0 ? bc.background_species : first;
            if (sp < 0) {
                *msg = "binary collisions: no neutral species";
                return PICGPU_INVALID_ARG;
            }
            const double T = bc.init_temperature > 0 ? bc.init_temperature : 293.15;
            const double d = bc.diameter[sp];
            smax = kPi * d * d * std::sqrt(2.0 * kKb * T / cfg.species[sp].mass);
        }
        std::vector<double> sm(nc, smax), r0(nc), r1(nc);
        for (int c = 0; c < nc; ++c) {
            r0[c] = host_uniform(cfg.seed, kStreamBinaryRemainder, uint32_t(c));
            r1[c] = host_uniform(cfg.seed, kStreamBinaryBgRemainder, uint32_t(c));
        }
        if (dmalloc(&st.bsmax, nc) || dmalloc(&st.brem, nc) || dmalloc(&st.bbgrem, nc)) {
            *msg = "binary collisions: device allocation failed";
            return PICGPU_OOM;
        }
        cudaMemcpyAsync(st.bsmax, sm.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st.brem, r0.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st.bbgrem, r1.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            *msg = "binary collisions: upload failed";
            return PICGPU_CUDA_ERROR;
        }
    }
    return PICGPU_OK;
}

void collide_free(CollideState& st) {
    void* ptrs[] = {st.svmax,      st.remainder,   st.xs,     st.xs32,     st.isvmax,   st.iremainder, st.ixs,
                    st.cell_start, st.cell_count,  st.cell_cursor, st.counts, st.scan_tmp, st.ncand,
                    st.cand_off,   st.stage,       st.flags,  st.pos,      st.stage_tmp, st.overflow,
                    st.iz_cell,    st.bsmax,       st.brem,   st.bbgrem,   st.blist,      st.boct,
                    st.psvmax,     st.premainder,  st.ipsvmax, st.ipremainder, st.n_live,
                    st.mspeed,     st.mstage,      st.mcount, st.moff,     st.mcounts,    st.mkin,
                    st.pstage,     st.pcount};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int s = 0; s < PICGPU_MAX_SPECIES; ++s) {
        if (st.ptab[s]) cudaFree(st.ptab[s]);
        if (st.idx[s]) cudaFree(st.idx[s]);
        if (st.sel[s]) cudaFree(st.sel[s]);
        if (st.sel2[s]) cudaFree(st.sel2[s]);
    }
    st = CollideState{};
}

// Cell occupancy of species s: st.idx[s] holds the particle indices grouped
// by cell; with `ordered` every cell's indices ascend (stable), otherwise
// their order within a cell follows the atomic scatter.
int occupancy(CollideState& st, const CollideArgs& a, int s, std::string* msg, int64_t* launches,
              bool ordered = true) {
    const int nc = a.m.n_cells;
    const long n = a.n[s];
    if (st.idx_cap[s] < n) {
        if (st.idx[s]) cudaFree(st.idx[s]);
        if (st.sel[s]) cudaFree(st.sel[s]);
        if (st.sel2[s]) cudaFree(st.sel2[s]);
        st.idx[s] = st.sel[s] = st.sel2[s] = nullptr;
        const long cap = std::max<long>(n + n / 4, 1024);
        if (dmalloc(&st.idx[s], cap) || dmalloc(&st.sel[s], cap) || dmalloc(&st.sel2[s], cap)) {
            *msg = "cell occupancy: device allocation failed";
            return PICGPU_OOM;
        }
        st.idx_cap[s] = cap;
    }
    int* cnt = st.cell_count + size_t(s) * (nc + 1);
    int* start = st.cell_start + size_t(s) * (nc + 1);
    cudaMemsetAsync(cnt, 0, (nc + 1) * sizeof(int), a.stream);
    cudaMemsetAsync(st.cell_cursor, 0, (nc + 1) * sizeof(int), a.stream);
    if (n > 0) {
        count_cells_kernel<<<grid_of(n, 256), 256, 0, a.stream>>>(a.sp[s].tet, int(n), cnt);
        *launches += 1;
    }
    exclusive_scan(cnt, start, nc, st.scan_tmp, a.stream, launches);
    if (n > 0) {
        scatter_cells_kernel<<<grid_of(n, 256), 256, 0, a.stream>>>(a.sp[s].tet, int(n), start, st.cell_cursor,
                                                                    st.idx[s]);
        *launches += 1;
        if (ordered) {
            order_cells_kernel<<<order_blocks(nc), 256, 0, a.stream>>>(nc, start, st.idx[s], st.sel[s]);
            *launches += 1;
        }
    }
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

namespace {

template <class R>
__global__ void permute_kernel(const int* __restrict__ idx, int total, DSpecies src, DSpecies dst) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x) {
        const int i = idx[j];
        dst.tet[j] = src.tet[i];
        if (sizeof(R) == 8) {
            for (int a = 0; a < 3; ++a) { dst.y64[a][j] = src.y64[a][i]; dst.u64[a][j] = src.u64[a][i]; }
        } else {
            for (int a = 0; a < 3; ++a) { dst.y32[a][j] = src.y32[a][i]; dst.u32[a][j] = src.u32[a][i]; }
        }
        if (src.nw) {
            dst.nw[j] = src.nw[i];
            dst.zq[j] = src.zq[i];
        }
    }
}

}  // namespace

int sort_species(CollideState& st, const DMesh& m, int s, const DSpecies& src, const DSpecies& dst, long n,
                 bool mixed, long* kept, cudaStream_t stream, std::string* msg, int64_t* launches) {
    const int nc = m.n_cells;
    if (!st.cell_start) {
        if (dmalloc(&st.cell_start, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) ||
            dmalloc(&st.cell_count, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) || dmalloc(&st.cell_cursor, nc + 1) ||
            dmalloc(&st.counts, kCollideCounts) || dmalloc(&st.scan_tmp, (nc + 1) / 1024 + 8)) {
            *msg = "cell sort: device allocation failed";
            return PICGPU_OOM;
        }
    }
    CollideArgs a{};
    a.m = m;
    a.stream = stream;
    a.sp[s] = src;
    a.n[s] = n;
    // the order inside a cell matters only where collisions pair particles by
    // list position; deposits are integer sums and the push is per particle
    const int e = occupancy(st, a, s, msg, launches, st.enabled != 0);
    if (e) return e;
    int total = 0;
    cudaMemcpyAsync(&total, st.cell_start + size_t(s) * (nc + 1) + nc, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess) {
        *msg = "cell sort failed";
        return PICGPU_CUDA_ERROR;
    }
    if (total > 0) {
        if (mixed) permute_kernel<float><<<grid_of(total, 256), 256, 0, stream>>>(st.idx[s], total, src, dst);
        else permute_kernel<double><<<grid_of(total, 256), 256, 0, stream>>>(st.idx[s], total, src, dst);
        *launches += 1;
    }
    *kept = total;
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

namespace {

PerezDev perez_setup(const CollideState& st, const CollideArgs& a, const CoulombSpecies& C) {
    PerezDev Z{};
    Z.ek = -1;
    for (int k = 0; k < PICGPU_MAX_SPECIES; ++k) Z.limit[k] = -1;
    if (!a.cfg->perez.enabled) return Z;
    for (int k = 0; k < C.n; ++k) {
        const int s = C.sp[k];
        if (s == a.cfg->electron_species) Z.ek = k;
        if (st.ptab[s]) {
            Z.limit[k] = st.plimit[s];
            Z.atomic[k] = st.patomic[s];
            Z.tab[k] = st.ptab[s];
        }
    }
    Z.on = Z.ek >= 0;
    Z.mE = a.cfg->species[a.cfg->electron_species].mass;
    Z.out = st.pstage;
    Z.n_out = st.pcount;
    Z.cap = st.pstage_cap;
    return Z;
}

void coulomb_setup(const CollideState& st, const CollideArgs& a, CoulombSpecies& C, CoulombParams& K) {
    const picgpu_config& cfg = *a.cfg;
    const int nc = a.m.n_cells;
    C = CoulombSpecies{};
    for (int s = 0; s < a.n_species; ++s) {
        if (cfg.species[s].charge == 0.0 || !cfg.species[s].solve_movement) continue;
        const int k = C.n++;
        C.sp[k] = s;
        C.m[k] = cfg.species[s].mass;
        C.q[k] = cfg.species[s].charge;
        C.w[k] = cfg.species[s].weight;
        C.start[k] = st.cell_start + size_t(s) * (nc + 1);
        C.idx[k] = st.idx[s];
        C.sel[k] = st.sel[s];
        C.sel2[k] = st.sel2[s];
        C.p[k] = a.sp[s];
    }
    K = CoulombParams{};
    K.n_cells = nc;
    K.vol = a.m.vol;
    K.cl = cfg.coulomb.coulomb_log;
    K.takizuka_abe = cfg.coulomb.pairing == PICGPU_PAIRING_TAKIZUKA_ABE;
    K.perez = cfg.coulomb.collide == PICGPU_COLLIDE_PEREZ;
    K.allow_intra = cfg.coulomb.allow_intra;
    K.calc_bmin = cfg.coulomb.calculate_bmin;
    K.debye_drift = cfg.coulomb.debye_drift;
    K.weight_corr = cfg.coulomb.weight_correction;
    K.dt = cfg.dt;
    K.seed = cfg.seed;
    K.step = uint32_t(a.step);
    K.counts = st.counts;
}

MccParams mcc_setup(const CollideState& st, const CollideArgs& a) {
    const picgpu_config& cfg = *a.cfg;
    const picgpu_mcc& mc = cfg.mcc;
    const int nc = a.m.n_cells;
    const int es = cfg.electron_species;
    MccParams M{};
    M.n_cells = nc;
    M.e_start = st.cell_start + size_t(es) * (nc + 1);
    M.e_idx = st.idx[es];
    M.svmax = st.svmax;
    M.rem = st.remainder;
    M.xs = st.xs;
    M.xs32 = st.xs32;
    M.n_xs = st.n_xs;
    M.n_gas = mc.gas_density;
    M.mg = mc.gas_mass;
    M.vth_gas = std::sqrt(kKb * mc.gas_temperature / mc.gas_mass);
    M.me = cfg.species[es].mass;
    M.me_c2_eV = float(M.me * kC * kC / 1.602176634e-19);
    M.dt = cfg.dt;
    for (int k = 0; k < 3; ++k) M.drift[k] = mc.gas_velocity[k];
    M.ex_th = mc.ex_threshold;
    M.iz_th = mc.iz_threshold;
    M.wEwN = cfg.species[es].weight / mc.gas_weight;
    M.wNwE = 1.0 / M.wEwN;
    M.create_e = mc.create_electron;
    M.create_i = mc.create_ion;
    M.relativistic = mc.scatter == 1;
    M.seed = cfg.seed;
    M.step = uint32_t(a.step);
    M.counts = st.counts;
    M.cand_off = st.cand_off;
    M.stage_cap = st.stage_cap;
    M.overflow = st.overflow;
    M.iz_cell = st.iz_cell;
    return M;
}

IonMccParams ion_setup(const CollideState& st, const CollideArgs& a) {
    const picgpu_config& cfg = *a.cfg;
    const picgpu_mcc& gas = cfg.mcc;
    const int nc = a.m.n_cells;
    const int is = cfg.ion_mcc.ion_species;
    IonMccParams M{};
    M.n_cells = nc;
    M.i_start = st.cell_start + size_t(is) * (nc + 1);
    M.i_idx = st.idx[is];
    M.svmax = st.isvmax;
    M.rem = st.iremainder;
    M.xs = st.ixs;
    M.n_xs = st.n_ixs;
    M.n_gas = gas.gas_density;
    M.mg = gas.gas_mass;
    M.vth_gas = std::sqrt(kKb * gas.gas_temperature / gas.gas_mass);
    M.mi = cfg.species[is].mass;
    M.dt = cfg.dt;
    for (int k = 0; k < 3; ++k) M.drift[k] = gas.gas_velocity[k];
    M.cx_th = cfg.ion_mcc.cx_threshold;
    M.seed = cfg.seed;
    M.step = uint32_t(a.step);
    M.counts = st.counts;
    return M;
}

__global__ void set_first_kernel(const int* n_dev, int* first_dev, int ns) {
    if (threadIdx.x < ns) first_dev[threadIdx.x] = n_dev[threadIdx.x];
}

// n += the secondaries just appended (clamped at the capacity).
__global__ void append_commit_kernel(int* n_dev, const int* add, long cap, int* overflow) {
    const long nn = long(*n_dev) + *add;
    if (nn > cap) {
        *overflow = 1;
        *n_dev = int(cap);
    } else {
        *n_dev = int(nn);
    }
}

}  // namespace

// The neutral species, the scratch lists and the launch of binary_kernel.
int launch_binary(CollideState& st, const CollideArgs& a, std::string* msg, int64_t* launches,
                  const unsigned* step_dev = nullptr) {
    const picgpu_config& cfg = *a.cfg;
    const picgpu_binary& bc = cfg.binary;
    const int nc = a.m.n_cells;
    BinaryParams B{};
    B.n_cells = nc;
    B.vol = a.m.vol;
    B.cell_class = a.m.cell_class;
    B.offset = a.m.offset;
    long need = 0;
    int sps[PICGPU_MAX_SPECIES];
    for (int s = 0; s < a.n_species; ++s) {
        if (cfg.species[s].charge != 0.0) continue;
        const int k = B.ns++;
        sps[k] = s;
        B.m[k] = cfg.species[s].mass;
        B.w[k] = cfg.species[s].weight;
        B.d[k] = bc.diameter[s];
        B.om[k] = bc.omega[s];
        B.start[k] = st.cell_start + size_t(s) * (nc + 1);
        B.idx[k] = st.idx[s];
        B.p[k] = a.sp[s];
        need += a.cap[s];
    }
    if (B.ns == 0) return PICGPU_OK;
    for (int k = 0; k < B.ns; ++k)
        for (int q = 0; q < B.ns; ++q) B.G[k][q] = std::exp(std::lgamma(2.5 - 0.5 * (B.om[k] + B.om[q])));
    if (st.bcap < need) {
        if (st.blist) cudaFree(st.blist);
        if (st.boct) cudaFree(st.boct);
        st.blist = st.boct = nullptr;
        if (dmalloc(&st.blist, need) || dmalloc(&st.boct, need)) {
            *msg = "binary collisions: device allocation failed";
            return PICGPU_OOM;
        }
        st.bcap = need;
    }
    B.vhs = bc.cross_section == PICGPU_XS_VARIABLE_HARD_SPHERE;
    B.weight_corr = bc.weight_correction;
    B.tref = bc.tref;
    B.smax = st.bsmax;
    B.rem = st.brem;
    B.bgrem = st.bbgrem;
    B.list = st.blist;
    B.oct = st.boct;
    B.dt = cfg.dt;
    B.seed = cfg.seed;
    B.step = uint32_t(a.step);
    B.step_dev = step_dev;
    B.counts = st.counts;
    const int bs = bc.background_species;
    if (bs >= 0 && cfg.mcc.gas_density > 0) {
        B.bg = 1;
        B.bg_n = cfg.mcc.gas_density;
        B.bg_T = cfg.mcc.gas_temperature;
        B.bg_m = cfg.species[bs].mass;
        B.bg_d = bc.diameter[bs];
        B.bg_om = bc.omega[bs];
        for (int q = 0; q < 3; ++q) B.bg_u[q] = cfg.mcc.gas_velocity[q];
        for (int k = 0; k < B.ns; ++k) B.Gbg[k] = std::exp(std::lgamma(2.5 - 0.5 * (B.om[k] + B.bg_om)));
    }
    (void)sps;
    if (a.mixed) binary_kernel<float><<<(nc + 63) / 64, 64, 0, a.stream>>>(B);
    else binary_kernel<double><<<(nc + 63) / 64, 64, 0, a.stream>>>(B);
    *launches += 1;
    return PICGPU_OK;
}

// Staging room for `total` candidates.
int ensure_stage(CollideState& st, long total, std::string* msg) {
    if (st.stage_cap >= total) return PICGPU_OK;
    if (st.stage) cudaFree(st.stage);
    if (st.flags) cudaFree(st.flags);
    if (st.pos) cudaFree(st.pos);
    if (st.stage_tmp) cudaFree(st.stage_tmp);
    st.stage = nullptr;
    st.flags = st.pos = st.stage_tmp = nullptr;
    const long cap = std::max<long>(total + total / 2, 4096);
    if (dmalloc(&st.stage, cap) || dmalloc(&st.flags, cap + 1) || dmalloc(&st.pos, cap + 2) ||
        dmalloc(&st.stage_tmp, cap / 1024 + 8)) {
        *msg = "MCC staging: device allocation failed";
        return PICGPU_OOM;
    }
    st.stage_cap = cap;
    return PICGPU_OK;
}

// Staged secondaries appended to the electron (bit 1) and ion (bit 2)
// species in (cell, candidate) order.
int append_stage(CollideState& st, const CollideArgs& a, int total, long newn[], std::string* msg,
                 int64_t* launches) {
    const picgpu_mcc& mc = a.cfg->mcc;
    const int es = a.cfg->electron_species;
    for (int bit = 1; bit <= 2; bit <<= 1) {
        const int s = bit == 1 ? es : mc.ion_species;
        if (s < 0 || (bit == 1 && !mc.create_electron) || (bit == 2 && !mc.create_ion)) continue;
        stage_flags_kernel<<<(total + 255) / 256, 256, 0, a.stream>>>(st.stage, total, bit, st.flags);
        exclusive_scan(st.flags, st.pos, total, st.stage_tmp, a.stream, launches);
        int add = 0;
        cudaMemcpyAsync(&add, st.pos + total, sizeof(int), cudaMemcpyDeviceToHost, a.stream);
        if (cudaStreamSynchronize(a.stream) != cudaSuccess) { *msg = "MCC: append failed"; return PICGPU_CUDA_ERROR; }
        *launches += 1;
        if (add == 0) continue;
        if (newn[s] + add > a.cap[s]) {
            *msg = "particle storage capacity exceeded by MCC secondaries (raise capacity_hint)";
            return PICGPU_CAPACITY;
        }
        if (a.mixed)
            stage_append_kernel<float><<<(total + 255) / 256, 256, 0, a.stream>>>(st.stage, total, bit, st.pos,
                                                                                 a.sp[s], int(newn[s]));
        else
            stage_append_kernel<double><<<(total + 255) / 256, 256, 0, a.stream>>>(st.stage, total, bit, st.pos,
                                                                                  a.sp[s], int(newn[s]));
        *launches += 1;
        newn[s] += add;
    }
    return PICGPU_OK;
}

// ElectronNeutralCollisionModel::performCollisions with the neutral parcels.
int mcc_parcels(CollideState& st, const CollideArgs& a, long newn[], std::string* msg, int64_t* launches) {
    const picgpu_config& cfg = *a.cfg;
    const picgpu_mcc& mc = cfg.mcc;
    const int nc = a.m.n_cells;
    const int es = cfg.electron_species, ns = mc.neutral_species;
    MccParcelParams M{};
    M.n_cells = nc;
    M.e_start = st.cell_start + size_t(es) * (nc + 1);
    M.e_idx = st.idx[es];
    M.n_start = st.cell_start + size_t(ns) * (nc + 1);
    M.n_idx = st.idx[ns];
    M.svmax = st.psvmax;
    M.rem = st.premainder;
    M.vol = a.m.vol;
    M.xs = st.xs;
    M.n_xs = st.n_xs;
    M.me = cfg.species[es].mass;
    M.mn = cfg.species[ns].mass;
    M.dt = cfg.dt;
    M.wE = cfg.species[es].weight;
    M.wN = cfg.species[ns].weight;
    M.wmax = std::max(M.wE, M.wN);
    M.ex_th = mc.ex_threshold;
    M.iz_th = mc.iz_threshold;
    M.create_e = mc.create_electron;
    M.create_i = mc.create_ion;
    M.relativistic = mc.scatter == 1;
    M.update_neutral = mc.keep_neutral_velocity ? 0 : 1;
    M.delete_neutral = mc.keep_neutrals ? 0 : 1;
    M.seed = cfg.seed;
    M.step = uint32_t(a.step);
    M.counts = st.counts;
    M.overflow = st.overflow;
    M.n_live = st.n_live;
    mcc_parcel_count_kernel<<<(nc + 255) / 256, 256, 0, a.stream>>>(M, st.ncand);
    exclusive_scan(st.ncand, st.cand_off, nc, st.scan_tmp, a.stream, launches);
    int total = 0;
    cudaMemcpyAsync(&total, st.cand_off + nc, sizeof(int), cudaMemcpyDeviceToHost, a.stream);
    if (cudaStreamSynchronize(a.stream) != cudaSuccess) { *msg = "MCC: candidate count failed"; return PICGPU_CUDA_ERROR; }
    int e = ensure_stage(st, total, msg);
    if (e) return e;
    M.cand_off = st.cand_off;
    M.stage_cap = st.stage_cap;
    if (a.mixed)
        mcc_parcel_kernel<float><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(
            M, a.sp[es], a.sp[ns], st.stage);
    else
        mcc_parcel_kernel<double><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(
            M, a.sp[es], a.sp[ns], st.stage);
    *launches += 2;
    if (total > 0 && (e = append_stage(st, a, total, newn, msg, launches))) return e;
    return PICGPU_OK;
}

// The electrons of the step's Perez ionisations: read back, put in key
// order and appended behind the electron store (room for them is the
// caller's: the store keeps an eighth of its size free for collision
// products).
int perez_append(CollideState& st, const CollideArgs& a, long newn[], long long* added, std::string* msg,
                 int64_t* launches) {
    const int es = a.cfg->electron_species;
    unsigned long long cnt = 0;
    if (cudaMemcpyAsync(&cnt, st.pcount, sizeof cnt, cudaMemcpyDeviceToHost, a.stream) != cudaSuccess ||
        cudaStreamSynchronize(a.stream) != cudaSuccess) {
        *msg = "Perez ionisation: reading the new electrons failed";
        return PICGPU_CUDA_ERROR;
    }
    *added = (long long)cnt;
    if (cnt == 0) return PICGPU_OK;
    if (cnt > (unsigned long long)st.pstage_cap) {
        *msg = "Perez ionisation: more new electrons in one step than the staging holds";
        return PICGPU_CAPACITY;
    }
    if (newn[es] + long(cnt) > a.cap[es]) {
        *msg = "Perez ionisation: the electron store has no room for the new electrons";
        return PICGPU_CAPACITY;
    }
    std::vector<PerezElectron> h(cnt);
    if (cudaMemcpyAsync(h.data(), st.pstage, cnt * sizeof(PerezElectron), cudaMemcpyDeviceToHost, a.stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(a.stream) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    std::sort(h.begin(), h.end(), [](const PerezElectron& x, const PerezElectron& y) { return x.key < y.key; });
    if (cudaMemcpyAsync(st.pstage, h.data(), cnt * sizeof(PerezElectron), cudaMemcpyHostToDevice, a.stream) !=
        cudaSuccess)
        return PICGPU_CUDA_ERROR;
    const int g = grid_of(long(cnt), 256);
    if (a.mixed) perez_append_kernel<float><<<g, 256, 0, a.stream>>>(st.pstage, long(cnt), a.sp[es], newn[es]);
    else perez_append_kernel<double><<<g, 256, 0, a.stream>>>(st.pstage, long(cnt), a.sp[es], newn[es]);
    *launches += 1;
    newn[es] += long(cnt);
    // the host copy must stay alive until the upload has run
    if (cudaStreamSynchronize(a.stream) != cudaSuccess) return PICGPU_CUDA_ERROR;
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

// The background MCC is the only reader of the cell lists this step.
bool mcc_lists_only(const picgpu_config& cfg) {
    return cfg.mcc.enabled && !cfg.mcc.neutral_parcels && !cfg.coulomb.enabled && !cfg.ion_mcc.enabled &&
           !cfg.binary.enabled;
}

int run_collisions(CollideState& st, const CollideArgs& a, int64_t counts[kCollideCounts], long newn[], int swapped[],
                   std::string* msg, int64_t* launches, double* phase_ms) {
    (void)phase_ms;
    const picgpu_config& cfg = *a.cfg;
    const int nc = a.m.n_cells;
    for (int s = 0; s < a.n_species; ++s) { newn[s] = a.n[s]; swapped[s] = 0; }
    cudaMemsetAsync(st.counts, 0, kCollideCounts * sizeof(unsigned long long), a.stream);
    long long perez_electrons = 0;
    // cell occupancy of every species (PICCloud::buildCellOccupancy); when
    // the background MCC alone reads the lists, only the cells with
    // candidates are put in index order (after the candidate count)
    const bool mcc_only = mcc_lists_only(cfg);
    for (int s = 0; s < a.n_species; ++s) {
        const int e = occupancy(st, a, s, msg, launches, !mcc_only);
        if (e) return e;
    }
    // Coulomb, electron-neutral, then ion-neutral (PICCloud::collisions,
    // PICCloud.C:526-539); parcels created on the way do not join the lists
    // (PICCloud::addNewParcel adds to the cloud only)
    if (cfg.coulomb.enabled) {
        CoulombSpecies C;
        CoulombParams K;
        coulomb_setup(st, a, C, K);
        const PerezDev Z = perez_setup(st, a, C);
        if (Z.on) cudaMemsetAsync(st.pcount, 0, sizeof(unsigned long long), a.stream);
        launch_coulomb(C, K, Z, a.mixed, a.stream);
        *launches += 1;
        if (Z.on) {
            const int e = perez_append(st, a, newn, &perez_electrons, msg, launches);
            if (e) return e;
        }
    }
    if (cfg.mcc.enabled && cfg.mcc.neutral_parcels) {
        const int e = mcc_parcels(st, a, newn, msg, launches);
        if (e) return e;
    }
    if (cfg.mcc.enabled) {
        const picgpu_mcc& mc = cfg.mcc;
        const int es = cfg.electron_species;
        MccParams M = mcc_setup(st, a);
        // candidates per cell and their staging offsets
        mcc_count_kernel<<<(nc + 255) / 256, 256, 0, a.stream>>>(M, st.ncand);
        if (mcc_only) {
            order_cells_kernel<<<order_blocks(nc), 256, 0, a.stream>>>(nc, M.e_start, st.idx[es], st.sel[es],
                                                                       st.ncand);
            *launches += 1;
        }
        exclusive_scan(st.ncand, st.cand_off, nc, st.scan_tmp, a.stream, launches);
        int total = 0;
        cudaMemcpyAsync(&total, st.cand_off + nc, sizeof(int), cudaMemcpyDeviceToHost, a.stream);
        if (cudaStreamSynchronize(a.stream) != cudaSuccess) { *msg = "MCC: candidate count failed"; return PICGPU_CUDA_ERROR; }
        if (st.stage_cap < total) {
            if (st.stage) cudaFree(st.stage);
            if (st.flags) cudaFree(st.flags);
            if (st.pos) cudaFree(st.pos);
            if (st.stage_tmp) cudaFree(st.stage_tmp);
            st.stage = nullptr; st.flags = st.pos = st.stage_tmp = nullptr;
            const long cap = std::max<long>(total + total / 2, 4096);
            if (dmalloc(&st.stage, cap) || dmalloc(&st.flags, cap + 1) || dmalloc(&st.pos, cap + 2) ||
                dmalloc(&st.stage_tmp, cap / 1024 + 8)) {
                *msg = "MCC staging: device allocation failed";
                return PICGPU_OOM;
            }
            st.stage_cap = cap;
        }
        M.cand_off = st.cand_off;
        M.stage_cap = st.stage_cap;
        M.overflow = st.overflow;
        M.iz_cell = st.iz_cell;
        if (a.mixed && !M.relativistic && M.xs32) launch_mcc_fp32(M, a.sp[es], st.stage, st.mcc_block, a.stream);
        else if (a.mixed) mcc_kernel<float><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[es], st.stage);
        else mcc_kernel<double><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[es], st.stage);
        *launches += 2;
        // append secondaries in (cell, candidate) order
        if (total > 0) {
            for (int bit = 1; bit <= 2; bit <<= 1) {
                const int s = bit == 1 ? es : mc.ion_species;
                if (s < 0 || (bit == 1 && !mc.create_electron) || (bit == 2 && !mc.create_ion)) continue;
                stage_flags_kernel<<<(total + 255) / 256, 256, 0, a.stream>>>(st.stage, total, bit, st.flags);
                exclusive_scan(st.flags, st.pos, total, st.stage_tmp, a.stream, launches);
                int add = 0;
                cudaMemcpyAsync(&add, st.pos + total, sizeof(int), cudaMemcpyDeviceToHost, a.stream);
                if (cudaStreamSynchronize(a.stream) != cudaSuccess) { *msg = "MCC: append failed"; return PICGPU_CUDA_ERROR; }
                *launches += 1;
                if (add == 0) continue;
                if (newn[s] + add > a.cap[s]) {
                    *msg = "particle storage capacity exceeded by MCC secondaries (raise capacity_hint)";
                    return PICGPU_CAPACITY;
                }
                if (a.mixed)
                    stage_append_kernel<float><<<(total + 255) / 256, 256, 0, a.stream>>>(st.stage, total, bit, st.pos,
                                                                                         a.sp[s], int(newn[s]));
                else
                    stage_append_kernel<double><<<(total + 255) / 256, 256, 0, a.stream>>>(
                        st.stage, total, bit, st.pos, a.sp[s], int(newn[s]));
                *launches += 1;
                newn[s] += add;
            }
        }
    }
    // ion-neutral last, over the ions present before this step's secondaries
    if (cfg.ion_mcc.enabled && cfg.ion_mcc.neutral_parcels) {
        const int is = cfg.ion_mcc.ion_species, ns = cfg.ion_mcc.neutral_species;
        IonParcelParams M{};
        M.n_cells = nc;
        M.i_start = st.cell_start + size_t(is) * (nc + 1);
        M.i_idx = st.idx[is];
        M.n_start = st.cell_start + size_t(ns) * (nc + 1);
        M.n_idx = st.idx[ns];
        M.svmax = st.ipsvmax;
        M.rem = st.ipremainder;
        M.vol = a.m.vol;
        M.xs = st.ixs;
        M.n_xs = st.n_ixs;
        M.mi = cfg.species[is].mass;
        M.mn = cfg.species[ns].mass;
        M.dt = cfg.dt;
        M.wI = cfg.species[is].weight;
        M.wN = cfg.species[ns].weight;
        M.wmax = std::max(M.wN, M.wI);
        M.cx_th = cfg.ion_mcc.cx_threshold;
        M.update_neutral = cfg.ion_mcc.keep_neutral_velocity ? 0 : 1;
        M.weight_corr = cfg.ion_mcc.weight_correction;
        M.seed = cfg.seed;
        M.step = uint32_t(a.step);
        M.counts = st.counts;
        // after electron - parcel collisions on the same neutral species the
        // lists hold only the neutrals that were not ionised and deleted
        // (sortedCellOccupancy is erased in place, ElectronNeutralCollisionModel.C:959-963)
        M.n_live = (cfg.mcc.enabled && cfg.mcc.neutral_parcels && cfg.mcc.neutral_species == ns) ? st.n_live : nullptr;
        if (a.mixed) ion_parcel_kernel<float><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[is], a.sp[ns]);
        else ion_parcel_kernel<double><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[is], a.sp[ns]);
        *launches += 1;
    }
    if (cfg.ion_mcc.enabled) {
        const int is = cfg.ion_mcc.ion_species;
        const IonMccParams M = ion_setup(st, a);
        if (a.mixed) ion_mcc_kernel<float><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[is]);
        else ion_mcc_kernel<double><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[is]);
        *launches += 1;
    }
    if (cfg.binary.enabled) {
        const int e = launch_binary(st, a, msg, launches);
        if (e) return e;
    }
    unsigned long long h[kCollideCounts];
    cudaMemcpyAsync(h, st.counts, sizeof h, cudaMemcpyDeviceToHost, a.stream);
    if (cudaStreamSynchronize(a.stream) != cudaSuccess) {
        *msg = "collision step failed";
        return PICGPU_CUDA_ERROR;
    }
    for (int k = 0; k < kCollideCounts; ++k) counts[k] = (int64_t)h[k];
    counts[21] = perez_electrons;
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

int collide_reserve_device(CollideState& st, const CollideArgs& a, std::string* msg) {
    const picgpu_config& cfg = *a.cfg;
    const int nc = a.m.n_cells;
    for (int s = 0; s < a.n_species; ++s) {
        if (st.idx_cap[s] >= a.cap[s]) continue;
        if (st.idx[s]) cudaFree(st.idx[s]);
        if (st.sel[s]) cudaFree(st.sel[s]);
        if (st.sel2[s]) cudaFree(st.sel2[s]);
        st.idx[s] = st.sel[s] = st.sel2[s] = nullptr;
        if (dmalloc(&st.idx[s], a.cap[s]) || dmalloc(&st.sel[s], a.cap[s]) || dmalloc(&st.sel2[s], a.cap[s])) {
            *msg = "cell occupancy: device allocation failed";
            return PICGPU_OOM;
        }
        st.idx_cap[s] = a.cap[s];
    }
    if (cfg.mcc.enabled) {
        // candidates per step: sum over cells of ceil(R + N_c n (sigma v)_max dt)
        // <= n_cells + N n (sigma v)_max dt; (sigma v)_max may grow, so twice
        // the initial bound plus margin
        const int es = cfg.electron_species;
        const double per = cfg.mcc.gas_density * st.svmax_init * cfg.dt;
        const long need = long(nc) + long(2.0 * per * double(a.cap[es])) + 65536;
        if (st.stage_cap < need) {
            if (st.stage) cudaFree(st.stage);
            if (st.flags) cudaFree(st.flags);
            if (st.pos) cudaFree(st.pos);
            if (st.stage_tmp) cudaFree(st.stage_tmp);
            st.stage = nullptr;
            st.flags = st.pos = st.stage_tmp = nullptr;
            if (dmalloc(&st.stage, need) || dmalloc(&st.flags, need + 1) || dmalloc(&st.pos, need + 2) ||
                dmalloc(&st.stage_tmp, need / 1024 + 8)) {
                *msg = "MCC staging: device allocation failed";
                return PICGPU_OOM;
            }
            st.stage_cap = need;
        }
    }
    return PICGPU_OK;
}

int run_collisions_device(CollideState& st, const CollideArgs& a, int* n_dev, int* first_dev,
                          const unsigned* step_dev, std::string* msg, int64_t* launches) {
    const picgpu_config& cfg = *a.cfg;
    const int nc = a.m.n_cells;
    set_first_kernel<<<1, 32, 0, a.stream>>>(n_dev, first_dev, a.n_species);
    *launches += 1;
    for (int s = 0; s < a.n_species; ++s) {
        if (st.idx_cap[s] < a.cap[s]) {
            *msg = "device-driven collisions: lists not reserved";
            return PICGPU_INVALID_ARG;
        }
        int* cnt = st.cell_count + size_t(s) * (nc + 1);
        int* start = st.cell_start + size_t(s) * (nc + 1);
        cudaMemsetAsync(cnt, 0, (nc + 1) * sizeof(int), a.stream);
        cudaMemsetAsync(st.cell_cursor, 0, (nc + 1) * sizeof(int), a.stream);
        const long cap = a.cap[s];
        count_cells_kernel<<<grid_of(cap, 256), 256, 0, a.stream>>>(a.sp[s].tet, int(cap), cnt, n_dev + s);
        exclusive_scan(cnt, start, nc, st.scan_tmp, a.stream, launches);
        scatter_cells_kernel<<<grid_of(cap, 256), 256, 0, a.stream>>>(a.sp[s].tet, int(cap), start, st.cell_cursor,
                                                                      st.idx[s], n_dev + s);
        *launches += 2;
        if (!mcc_lists_only(cfg)) {
            order_cells_kernel<<<order_blocks(nc), 256, 0, a.stream>>>(nc, start, st.idx[s], st.sel[s]);
            *launches += 1;
        }
    }
    if (cfg.coulomb.enabled) {
        CoulombSpecies C;
        CoulombParams K;
        coulomb_setup(st, a, C, K);
        K.step_dev = step_dev;
        PerezDev Z{};
        Z.ek = -1;
        launch_coulomb(C, K, Z, a.mixed, a.stream);
        *launches += 1;
    }
    if (cfg.mcc.enabled) {
        const picgpu_mcc& mc = cfg.mcc;
        const int es = cfg.electron_species;
        MccParams M = mcc_setup(st, a);
        M.step_dev = step_dev;
        const long scap = st.stage_cap;
        mcc_count_kernel<<<(nc + 255) / 256, 256, 0, a.stream>>>(M, st.ncand);
        if (mcc_lists_only(cfg)) {
            order_cells_kernel<<<order_blocks(nc), 256, 0, a.stream>>>(nc, M.e_start, st.idx[es], st.sel[es],
                                                                       st.ncand);
            *launches += 1;
        }
        exclusive_scan(st.ncand, st.cand_off, nc, st.scan_tmp, a.stream, launches);
        if (a.mixed && !M.relativistic && M.xs32) launch_mcc_fp32(M, a.sp[es], st.stage, st.mcc_block, a.stream);
        else if (a.mixed) mcc_kernel<float><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[es], st.stage);
        else mcc_kernel<double><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[es], st.stage);
        *launches += 2;
        for (int bit = 1; bit <= 2; bit <<= 1) {
            const int s = bit == 1 ? es : mc.ion_species;
            if (s < 0 || (bit == 1 && !mc.create_electron) || (bit == 2 && !mc.create_ion)) continue;
            // slots past the staged candidates (cand_off[nc]) are flagged 0
            stage_flags_kernel<<<unsigned((scap + 255) / 256), 256, 0, a.stream>>>(st.stage, int(scap), bit, st.flags,
                                                                                   st.cand_off + nc);
            exclusive_scan(st.flags, st.pos, scap, st.stage_tmp, a.stream, launches);
            if (a.mixed)
                stage_append_kernel<float><<<unsigned((scap + 255) / 256), 256, 0, a.stream>>>(
                    st.stage, int(scap), bit, st.pos, a.sp[s], 0, n_dev + s, a.cap[s], st.overflow);
            else
                stage_append_kernel<double><<<unsigned((scap + 255) / 256), 256, 0, a.stream>>>(
                    st.stage, int(scap), bit, st.pos, a.sp[s], 0, n_dev + s, a.cap[s], st.overflow);
            append_commit_kernel<<<1, 1, 0, a.stream>>>(n_dev + s, st.pos + scap, a.cap[s], st.overflow);
            *launches += 3;
        }
    }
    if (cfg.ion_mcc.enabled) {
        const int is = cfg.ion_mcc.ion_species;
        IonMccParams M = ion_setup(st, a);
        M.step_dev = step_dev;
        if (a.mixed) ion_mcc_kernel<float><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[is]);
        else ion_mcc_kernel<double><<<(nc + st.mcc_block - 1) / st.mcc_block, st.mcc_block, 0, a.stream>>>(M, a.sp[is]);
        *launches += 1;
    }
    if (cfg.binary.enabled) {
        const int e = launch_binary(st, a, msg, launches, step_dev);
        if (e) return e;
    }
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

// ------------------------------------------------------- PairMerging ---
namespace {

struct MergeParams {
    int n_cells;
    DMesh m;
    const int* start;          // cell occupancy of the species
    const int* idx;
    int* sel;                  // scratch: mergeSelect per cell (same layout as idx)
    double* speed;             // scratch: |U| per list position
    DSpecies p;
    double w, mass;
    int li;                    // entry of the merge list (random stream)
    double n_dev, reduction, cos_angle, velocity_ratio;
    int cell_max, max_checks, n_check, max_per_cell;
    uint64_t seed;
    uint32_t step;
    MergedParcel* stage;       // cell c stages from start[c] / 2 on
    int* count;                // merges per cell
    unsigned long long* counts;  // merged, checked
    double* kin;
};

template <class R>
__device__ __forceinline__ double mw(const MergeParams& M, int i) {
    return M.p.nw ? M.p.nw[i] : M.w;
}

// The parcel's position: cell centre plus its tet's face-triangle offsets
// weighted by the barycentric coordinates 1..3 (the oracle's position()).
template <class R>
__device__ void parcel_position(const MergeParams& M, int i, double* x) {
    const int tg = M.p.tet[i];
    const int c = tg / 12, t = tg - 12 * c;
    const double* off = M.m.offset + size_t(M.m.cell_class[c]) * 24;
    double y[3];
    for (int a = 0; a < 3; ++a) y[a] = sizeof(R) == 8 ? M.p.y64[a][i] : double(M.p.y32[a][i]);
    for (int a = 0; a < 3; ++a)
        x[a] = M.m.cc[3 * size_t(c) + a] + y[0] * off[3 * c_tetC.tri[t][0] + a] +
               y[1] * off[3 * c_tetC.tri[t][1] + a] + y[2] * off[3 * c_tetC.tri[t][2] + a];
}

// x in cell c: the tet whose smallest barycentric coordinate is largest,
// coordinates clamped to >= 0 and renormalised (mesh locate within a known
// cell).  Returns the tet index cell 12 + t.
__device__ int locate_in_cell(const DMesh& m, int c, const double* x, double* y) {
    const double r[3] = {x[0] - m.cc[3 * size_t(c)], x[1] - m.cc[3 * size_t(c) + 1], x[2] - m.cc[3 * size_t(c) + 2]};
    int best = 0;
    double best_min = -1e300, q[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 12; ++t) {
        const double* row = m.tetinv + (size_t(m.cell_class[c]) * 12 + t) * 9;
        double w[3];
        for (int k = 0; k < 3; ++k) w[k] = row[3 * k] * r[0] + row[3 * k + 1] * r[1] + row[3 * k + 2] * r[2];
        const double lowest = fmin(fmin(1.0 - w[0] - w[1] - w[2], w[0]), fmin(w[1], w[2]));
        if (lowest > best_min) {
            best_min = lowest;
            best = t;
            q[0] = w[0];
            q[1] = w[1];
            q[2] = w[2];
        }
    }
    const double all[4] = {fmax(1.0 - q[0] - q[1] - q[2], 0.0), fmax(q[0], 0.0), fmax(q[1], 0.0), fmax(q[2], 0.0)};
    const double sum = all[0] + all[1] + all[2] + all[3];
    for (int k = 0; k < 3; ++k) y[k] = all[k + 1] / sum;
    return 12 * c + best;
}

// Heap sort of sel[0, n) by (key[sel], sel): the ascending speed order of
// PairMerging.C:110-113, ties by list position.
__device__ __forceinline__ bool merge_less(const double* key, int a, int b) {
    return key[a] < key[b] || (key[a] == key[b] && a < b);
}
__device__ void sift_down(int* sel, const double* key, int root, int n) {
    while (true) {
        int child = 2 * root + 1;
        if (child >= n) return;
        if (child + 1 < n && merge_less(key, sel[child], sel[child + 1])) ++child;
        if (!merge_less(key, sel[root], sel[child])) return;
        const int t = sel[root];
        sel[root] = sel[child];
        sel[child] = t;
        root = child;
    }
}
__device__ void heap_sort(int* sel, const double* key, int n) {
    for (int k = n / 2 - 1; k >= 0; --k) sift_down(sel, key, k, n);
    for (int e = n - 1; e > 0; --e) {
        const int t = sel[0];
        sel[0] = sel[e];
        sel[e] = t;
        sift_down(sel, key, 0, e);
    }
}

// PairMerging::mergeParticles (PairMerging.C:71-259) for one cell, one
// thread per cell, with the reference's quirks: the speeds of the
// acceptance tests are those of the LIST positions pId1 / pId2 (not of the
// parcels they select, and not shifted after a merge), a well-aligned pair
// (velocity angle below angleDifference) is rejected, and the merged parcel
// gets charge modifier 1 (PICCloud::addNewParcel).
template <class R>
__global__ void merge_kernel(MergeParams M) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    const int s0 = M.start[c];
    int N = M.start[c + 1] - s0;
    int merged = 0;
    if (N <= M.cell_max) {
        M.count[c] = 0;
        return;
    }
    const int* L = M.idx + s0;
    int* sel = M.sel + s0;
    double* speed = M.speed + s0;
    int nTarget = int(double(N) * M.reduction);
    if (N - nTarget > M.max_per_cell) nTarget = N - M.max_per_cell;
    for (int k = 0; k < N; ++k) {
        const int i = L[k];
        double U[3];
        for (int a = 0; a < 3; ++a) U[a] = sizeof(R) == 8 ? M.p.u64[a][i] : double(M.p.u32[a][i]);
        speed[k] = sqrt(U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
        sel[k] = k;
    }
    heap_sort(sel, speed, N);
    Philox rng(M.seed, kStreamMerge | uint32_t(M.li), uint32_t(c), M.step);
    MergedParcel* out = M.stage + s0 / 2;
    unsigned long long checked = 0;
    double kin = 0.0;
    int checks = 0;
    while (N > nTarget) {
        int pId1 = int(rng.uniform() * double(N));
        if (pId1 >= N) pId1 = N - 1;
        const int i1 = L[sel[pId1]];
        int pId2 = pId1 - M.n_check / 2;
        if (pId2 < 0) pId2 = 0;
        if (pId2 + M.n_check > N - 1) pId2 = N - M.n_check - 1;
        if (pId2 < 0) pId2 = 0;
        int found = -1;
        for (int k = 0; k < M.n_check; ++k) {
            if (pId2 == pId1) pId2++;
            if (pId2 >= N) break;
            const int i2 = L[sel[pId2]];
            checked++;
            if (M.n_dev - fabs(mw<R>(M, i2) - mw<R>(M, i1)) < 0.0) { pId2++; continue; }
            if ((M.p.zq ? M.p.zq[i2] : 1) != (M.p.zq ? M.p.zq[i1] : 1)) { pId2++; continue; }
            double U1[3], U2[3];
            for (int a = 0; a < 3; ++a) {
                U1[a] = sizeof(R) == 8 ? M.p.u64[a][i1] : double(M.p.u32[a][i1]);
                U2[a] = sizeof(R) == 8 ? M.p.u64[a][i2] : double(M.p.u32[a][i2]);
            }
            if (U2[0] * U1[0] + U2[1] * U1[1] + U2[2] * U1[2] > speed[pId2] * speed[pId1] * M.cos_angle) {
                pId2++;
                continue;
            }
            double ratio = speed[pId2] / speed[pId1];
            if (ratio > 1.0) ratio = 1.0 / ratio;
            if (ratio < M.velocity_ratio) { pId2++; continue; }
            found = pId2;
            break;
        }
        if (found >= 0) {
            pId2 = found;
            const int i2 = L[sel[pId2]];
            const double n1 = mw<R>(M, i1), n2 = mw<R>(M, i2);
            const double nSum = n1 + n2;
            double x1[3], x2[3], U1[3], U2[3], com[3], nU[3];
            parcel_position<R>(M, i1, x1);
            parcel_position<R>(M, i2, x2);
            for (int a = 0; a < 3; ++a) {
                U1[a] = sizeof(R) == 8 ? M.p.u64[a][i1] : double(M.p.u32[a][i1]);
                U2[a] = sizeof(R) == 8 ? M.p.u64[a][i2] : double(M.p.u32[a][i2]);
                com[a] = (n1 * x1[a] + n2 * x2[a]) / nSum;
                nU[a] = (n1 * U1[a] + n2 * U2[a]) / nSum;
            }
            const double pre = 0.5 * M.mass *
                               ((U1[0] * U1[0] + U1[1] * U1[1] + U1[2] * U1[2]) * n1 +
                                (U2[0] * U2[0] + U2[1] * U2[1] + U2[2] * U2[2]) * n2);
            const double post = 0.5 * M.mass * (nU[0] * nU[0] + nU[1] * nU[1] + nU[2] * nU[2]) * nSum;
            kin += post - pre;
            MergedParcel& mp = out[merged++];
            mp.tet = locate_in_cell(M.m, c, com, mp.y);
            for (int a = 0; a < 3; ++a) mp.U[a] = nU[a];
            mp.nw = nSum;
            M.p.tet[i1] = -1;
            M.p.tet[i2] = -1;
            const int minPos = min(pId1, pId2), maxPos = max(pId1, pId2);
            for (int k = minPos; k < N - 2; ++k) sel[k] = k >= maxPos - 1 ? sel[k + 2] : sel[k + 1];
            N -= 2;
        }
        checks++;
        if (checks > M.max_checks) break;
    }
    M.count[c] = merged;
    if (merged) atomicAdd(M.counts, (unsigned long long)merged);
    if (checked) atomicAdd(M.counts + 1, checked);
    if (kin != 0.0) atomicAdd(M.kin, kin);
}

template <class R>
__global__ void merge_append_kernel(int n_cells, const int* __restrict__ start, const int* __restrict__ count,
                                    const int* __restrict__ off, const MergedParcel* __restrict__ stage, DSpecies p,
                                    long first) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    const MergedParcel* src = stage + start[c] / 2;
    for (int k = 0; k < count[c]; ++k) {
        const long j = first + off[c] + k;
        const MergedParcel& mp = src[k];
        p.tet[j] = mp.tet;
        for (int a = 0; a < 3; ++a) {
            if (sizeof(R) == 8) {
                p.y64[a][j] = mp.y[a];
                p.u64[a][j] = mp.U[a];
            } else {
                p.y32[a][j] = float(mp.y[a]);
                p.u32[a][j] = float(mp.U[a]);
            }
        }
        p.nw[j] = mp.nw;
        p.zq[j] = 1;
    }
}

}  // namespace

int merge_select(CollideState& st, const CollideArgs& a, int li, int s, long long* total, std::string* msg,
                 int64_t* launches) {
    const picgpu_merging& mg = a.cfg->merging;
    const int nc = a.m.n_cells;
    *total = 0;
    int e = occupancy(st, a, s, msg, launches);
    if (e) return e;
    const long n = a.n[s];
    if (st.mspeed_cap < std::max<long>(n, 1) || !st.mcount) {
        if (st.mspeed) cudaFree(st.mspeed);
        if (st.mstage) cudaFree(st.mstage);
        st.mspeed = nullptr;
        st.mstage = nullptr;
        const long cap = std::max<long>(n + n / 4, 1024);
        if (dmalloc(&st.mspeed, cap) || dmalloc(&st.mstage, cap / 2 + 1) ||
            (!st.mcount && (dmalloc(&st.mcount, nc + 1) || dmalloc(&st.moff, nc + 1) || dmalloc(&st.mcounts, 2) ||
                            dmalloc(&st.mkin, 1)))) {
            *msg = "merging: device allocation failed";
            return PICGPU_OOM;
        }
        st.mspeed_cap = cap;
        st.mstage_cap = cap / 2 + 1;
        cudaMemsetAsync(st.mcounts, 0, 2 * sizeof(unsigned long long), a.stream);
        cudaMemsetAsync(st.mkin, 0, sizeof(double), a.stream);
    }
    MergeParams M{};
    M.n_cells = nc;
    M.m = a.m;
    M.start = st.cell_start + size_t(s) * (nc + 1);
    M.idx = st.idx[s];
    M.sel = st.sel[s];
    M.speed = st.mspeed;
    M.p = a.sp[s];
    M.w = a.cfg->species[s].weight;
    M.mass = a.cfg->species[s].mass;
    M.li = li;
    M.n_dev = mg.n_deviation[li];
    M.reduction = mg.reduction_factor;
    M.cos_angle = std::cos(mg.angle_difference * 3.14159265358979323846 / 180.0);
    M.velocity_ratio = mg.velocity_ratio;
    M.cell_max = mg.cell_parcels_max;
    M.max_checks = mg.max_checks;
    M.n_check = mg.n_check_neighbors;
    M.max_per_cell = mg.merge_maximum_per_cell;
    M.seed = a.cfg->seed;
    M.step = uint32_t(a.step);
    M.stage = st.mstage;
    M.count = st.mcount;
    M.counts = st.mcounts;
    M.kin = st.mkin;
    if (a.mixed) merge_kernel<float><<<(nc + 127) / 128, 128, 0, a.stream>>>(M);
    else merge_kernel<double><<<(nc + 127) / 128, 128, 0, a.stream>>>(M);
    exclusive_scan(st.mcount, st.moff, nc, st.scan_tmp, a.stream, launches);
    *launches += 1;
    int t = 0;
    if (cudaMemcpyAsync(&t, st.moff + nc, sizeof(int), cudaMemcpyDeviceToHost, a.stream) != cudaSuccess ||
        cudaStreamSynchronize(a.stream) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    *total = t;
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

int merge_append(CollideState& st, const CollideArgs& a, int s, long first, long long total, std::string* msg,
                 int64_t* launches) {
    (void)msg;
    if (total <= 0) return PICGPU_OK;
    const int nc = a.m.n_cells;
    const int* start = st.cell_start + size_t(s) * (nc + 1);
    if (a.mixed)
        merge_append_kernel<float><<<(nc + 255) / 256, 256, 0, a.stream>>>(nc, start, st.mcount, st.moff, st.mstage,
                                                                          a.sp[s], first);
    else
        merge_append_kernel<double><<<(nc + 255) / 256, 256, 0, a.stream>>>(nc, start, st.mcount, st.moff, st.mstage,
                                                                           a.sp[s], first);
    *launches += 1;
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

int merge_counters(CollideState& st, cudaStream_t s, long long* merged, long long* checked, double* kin_err) {
    *merged = *checked = 0;
    *kin_err = 0.0;
    if (!st.mcounts) return PICGPU_OK;
    unsigned long long h[2];
    double k = 0.0;
    if (cudaMemcpyAsync(h, st.mcounts, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&k, st.mkin, sizeof k, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    cudaMemsetAsync(st.mcounts, 0, 2 * sizeof(unsigned long long), s);
    cudaMemsetAsync(st.mkin, 0, sizeof(double), s);
    *merged = (long long)h[0];
    *checked = (long long)h[1];
    *kin_err = k;
    return PICGPU_OK;
}


}  // namespace pgd
