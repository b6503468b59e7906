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
//                    (cell, candidate) order
//   coulomb_*        NanbuYonemuraPairing::pairANDcollide (NanbuYonemuraPairing.C:56-325)
//                    with NanbuCollision::collide (NanbuCollision.C:60-161),
//                    one thread per cell
// The collision arithmetic is FP64 for both particle forms.
#include <algorithm>
#include <vector>

#include "collide.h"

namespace pgd {

__constant__ TetConst c_tetC;

namespace {

constexpr double kEch = 1.602176634e-19;
constexpr double kKb = 1.380649e-23;
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
__global__ void count_cells_kernel(const int32_t* __restrict__ tet, int n, int* __restrict__ count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = tet[i];
        if (t >= 0) atomicAdd(count + t / 12, 1);
    }
}

__global__ void scatter_cells_kernel(const int32_t* __restrict__ tet, int n, const int* __restrict__ start,
                                     int* __restrict__ cursor, int* __restrict__ idx) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = tet[i];
        if (t >= 0) {
            const int c = t / 12;
            idx[start[c] + atomicAdd(cursor + c, 1)] = i;
        }
    }
}

// Order every cell's list by particle index (insertion sort; lists are short).
__global__ void order_cells_kernel(int n_cells, const int* __restrict__ start, int* __restrict__ idx) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    int* a = idx + start[c];
    const int L = start[c + 1] - start[c];
    for (int k = 1; k < L; ++k) {
        const int v = a[k];
        int j = k - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            --j;
        }
        a[j + 1] = v;
    }
}

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

// List cross section, linear between bracketing nodes, end values held
// (ListCrossSection.C:33-88).
__device__ double interp_xs(double x, const double* e, const double* v, int n) {
    if (x <= e[0]) return v[0];
    if (x >= e[n - 1]) return v[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] <= x) lo = mid; else hi = mid;
    }
    if (e[lo] == x) return v[lo];
    return v[lo] + ((x - e[lo]) / (e[hi] - e[lo])) * (v[hi] - v[lo]);
}

struct MccParams {
    int n_cells;
    const int* e_start;   // n_cells + 1
    const int* e_idx;
    double* svmax;
    double* rem;
    const double* xs;     // 4 x n_xs
    int n_xs;
    double n_gas, vth_gas, mg, me, dt;
    double drift[3];
    double ex_th, iz_th;
    double wEwN, wNwE;
    int create_e, create_i;
    uint64_t seed;
    uint32_t step;
    const int* cand_off;  // n_cells + 1
    unsigned long long* counts;
};

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
    Rng r(M.seed, kStreamMcc, uint32_t(c), M.step);
    unsigned long long nel = 0, nex = 0, niz = 0;
    const int base = M.cand_off[c];
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
        const double Qel = interp_xs(eV, E, EL, M.n_xs);
        const double Qex = interp_xs(eV, E, EX, M.n_xs);
        const double Qiz = interp_xs(eV, E, IZ, M.n_xs);
        const double Qt = Qel + Qex + Qiz;
        if (Qt * cR > M.svmax[c]) M.svmax[c] = Qt * cR;
        const double Ru = r.uniform();
        if (Ru <= Qel / sigmaT) {
            nel++;
            nanbu_scatter(eV, Ue, Un, M.me, M.mg, r);
            Vel<R>::put(el, pi, Ue);
        } else if (eV >= M.ex_th && Ru <= (Qel + Qex) / sigmaT) {
            nex++;
            const double f = sqrt(1.0 - M.ex_th / eV);
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= M.ex_th;
            nanbu_scatter(eV, Ue, Un, M.me, M.mg, r);
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
            nanbu_scatter(eV, Ue, Un, M.me, M.mg, r);
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
                nanbu_scatter(Ep, ne, un2, M.me, M.mg, r);
                sc.flag |= 1;
                sc.ue[0] = ne.x; sc.ue[1] = ne.y; sc.ue[2] = ne.z;
            }
            if (sc.flag) {
                sc.tet = el.tet[pi];
                if (el.y64[0]) { sc.y[0] = el.y64[0][pi]; sc.y[1] = el.y64[1][pi]; sc.y[2] = el.y64[2][pi]; }
                else { sc.y[0] = el.y32[0][pi]; sc.y[1] = el.y32[1][pi]; sc.y[2] = el.y32[2][pi]; }
            }
            stage[base + i] = sc;
            continue;
        }
        stage[base + i].flag = 0;
    }
    atomicAdd(M.counts + 0, (unsigned long long)nC);
    if (nel) atomicAdd(M.counts + 1, nel);
    if (nex) atomicAdd(M.counts + 2, nex);
    if (niz) atomicAdd(M.counts + 3, niz);
}

__global__ void stage_flags_kernel(const Secondary* __restrict__ stage, int n, int bit, int* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = (stage[i].flag & bit) ? 1 : 0;
}

template <class R>
__global__ void stage_append_kernel(const Secondary* __restrict__ stage, int n, int bit,
                                    const int* __restrict__ pos, DSpecies dst, int base) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(stage[i].flag & bit)) return;
    const int k = base + pos[i];
    const Secondary& s = stage[i];
    dst.tet[k] = s.tet;
    const double* u = bit == 1 ? s.ue : s.ui;
    if (dst.y64[0]) {
        for (int a = 0; a < 3; ++a) { dst.y64[a][k] = s.y[a]; dst.u64[a][k] = u[a]; }
    } else {
        for (int a = 0; a < 3; ++a) { dst.y32[a][k] = float(s.y[a]); dst.u32[a][k] = float(u[a]); }
    }
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

template <class R>
__device__ void collide(const CoulombSpecies& C, int a, int ia, int b, int ib, double nP, double nQ, double nPQ,
                        double cl, double dt, Rng& r) {
    const double mP = C.m[a], qP = C.q[a], mQ = C.m[b], qQ = C.q[b];
    V3d UP = Vel<R>::get(C.p[a], ia), UQ = Vel<R>::get(C.p[b], ib);
    const double reMass = mP * mQ / (mP + mQ);
    const V3d g = {UP.x - UQ.x, UP.y - UQ.y, UP.z - UQ.z};
    const double gm = magd(g);
    const double A = qP * qQ / (eps0c() * reMass);
    const double s = cl / (4.0 * kPi) * (A * A) * (nQ * nP / nPQ) * (1.0 / (gm * gm * gm)) * dt;
    const double cosChi = cos_chi(s, r);
    const double sinChi = sqrt(1.0 - cosChi * cosChi);
    const double gp = sqrt(g.y * g.y + g.z * g.z);
    const double eps = 2.0 * kPi * r.uniform();
    const double ce = cos(eps), se = sin(eps);
    const V3d h = {gp * ce, -1.0 * (g.y * g.x * ce + gm * g.z * se) / gp, -1.0 * (g.z * g.x * ce - gm * g.y * se) / gp};
    const V3d d = {(1.0 - cosChi) * g.x + sinChi * h.x, (1.0 - cosChi) * g.y + sinChi * h.y,
                   (1.0 - cosChi) * g.z + sinChi * h.z};
    const double kp = mQ / (mP + mQ), kq = mP / (mP + mQ);
    Vel<R>::put(C.p[a], ia, V3d{UP.x - kp * d.x, UP.y - kp * d.y, UP.z - kp * d.z});
    Vel<R>::put(C.p[b], ib, V3d{UQ.x + kq * d.x, UQ.y + kq * d.y, UQ.z + kq * d.z});
}

__device__ void shuffle(int* a, int n, Rng& r) {
    for (int k = n - 1; k > 0; --k) {
        int j = int(r.uniform() * double(k + 1));
        if (j > k) j = k;
        const int t = a[k]; a[k] = a[j]; a[j] = t;
    }
}

template <class R>
__global__ void coulomb_kernel(CoulombSpecies C, int n_cells, const double* __restrict__ vol, double cl,
                               int allow_intra, double dt, uint64_t seed, uint32_t step,
                               unsigned long long* counts) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    const double V = vol[c];
    Rng r(seed, kStreamCoulomb, uint32_t(c), step);
    unsigned long long pairs = 0;
    for (int i = 0; i < C.n; ++i) {
        for (int jj = C.n - 1; jj >= i; --jj) {
            const int a = i, b = jj;
            const int sa = C.start[a][c], sb = C.start[b][c];
            const int nA = C.start[a][c + 1] - sa, nB = C.start[b][c + 1] - sb;
            const int* LA = C.idx[a] + sa;
            const int* LB = C.idx[b] + sb;
            const double sA = double(nA) * C.w[a];
            const double sB = a != b ? double(nB) * C.w[b] : 0.0;
            if (a == b && nA > 1) {
                if (!allow_intra) continue;
                int* sel = C.sel[a] + sa;
                for (int k = 0; k < nA; ++k) sel[k] = k;
                shuffle(sel, nA, r);
                const double n = sA / V;
                if (nA % 2 != 0) {
                    double nAA = 2.0 * C.w[a];
                    for (int x = 0; x < nA - 2; x += 2) nAA += 2.0 * C.w[a];
                    const double n12 = nAA / V;
                    for (int x = 0; x < nA - 2; x += 2)
                        collide<R>(C, a, LA[sel[x]], a, LA[sel[x + 1]], n, n, n12, cl, dt, r);
                    collide<R>(C, a, LA[sel[nA - 1]], a, LA[sel[0]], n, n, n12, cl, dt, r);
                    pairs += 1 + nA / 2;
                } else {
                    double nAA = 0.0;
                    for (int x = 0; x < nA - 1; x += 2) nAA += 2.0 * C.w[a];
                    const double n12 = nAA / V;
                    for (int x = 0; x < nA - 1; x += 2)
                        collide<R>(C, a, LA[sel[x]], a, LA[sel[x + 1]], n, n, n12, cl, dt, r);
                    pairs += nA / 2;
                }
            } else if (a != b && min(nA, nB) != 0) {
                const double wmin = fmin(C.w[a], C.w[b]);
                if (nA == nB) {
                    const double nP = sA / V, nQ = sB / V;
                    int* sel = C.sel[a] + sa;
                    for (int k = 0; k < nA; ++k) sel[k] = k;
                    shuffle(sel, nA, r);
                    double nAB = 0.0;
                    for (int k = 0; k < nA; ++k) nAB += wmin;
                    const double nPQ = nAB / V;
                    for (int k = 0; k < nA; ++k)
                        collide<R>(C, a, LA[sel[k]], b, LB[sel[nA - k - 1]], nP, nQ, nPQ, cl, dt, r);
                    pairs += nA;
                } else {
                    const bool aMin = nA < nB;
                    const int minS = aMin ? a : b, maxS = aMin ? b : a;
                    const int* Lmin = aMin ? LA : LB;
                    const int* Lmax = aMin ? LB : LA;
                    const int nMax = max(nA, nB), nMin = min(nA, nB);
                    int* smin = C.sel[minS] + (aMin ? sa : sb);
                    int* smax = C.sel2[maxS] + (aMin ? sb : sa);
                    for (int k = 0; k < nMax; ++k) { smax[k] = k; if (k < nMin) smin[k] = k; }
                    shuffle(smin, nMin, r);
                    shuffle(smax, nMax, r);
                    const double nMaxS = (maxS == a ? sA : sB) / V;
                    const double nMinS = (maxS == a ? sB : sA) / V;
                    double nAB = 0.0;
                    for (int l = 0; l < nMax; ++l) nAB += wmin;
                    const double n12 = nAB / V;
                    int k = 0;
                    for (int l = 0; l < nMax; ++l) {
                        if (k >= nMin) k = 0;
                        collide<R>(C, maxS, Lmax[smax[l]], minS, Lmin[smin[k]], nMaxS, nMinS, n12, cl, dt, r);
                        ++k;
                    }
                    pairs += nMax;
                }
            }
        }
    }
    if (pairs) atomicAdd(counts + 4, pairs);
}

template <class T>
cudaError_t dmalloc(T** p, size_t n) {
    return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T));
}

int grid_of(long n, int bs) { return int(std::max<long>(1, std::min<long>((n + bs - 1) / bs, 148L * 16))); }

}  // namespace

cudaError_t collide_set_tables(const TetConst& t) { return cudaMemcpyToSymbol(c_tetC, &t, sizeof t); }

int collide_init(CollideState& st, const picgpu_config& cfg, const DMesh& m, cudaStream_t s, std::string* msg) {
    st.enabled = cfg.mcc.enabled || cfg.coulomb.enabled;
    if (!st.enabled) return PICGPU_OK;
    const int nc = m.n_cells;
    if (dmalloc(&st.cell_start, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) ||
        dmalloc(&st.cell_count, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) || dmalloc(&st.cell_cursor, nc + 1) ||
        dmalloc(&st.counts, 8) || dmalloc(&st.scan_tmp, (nc + 1) / 1024 + 8)) {
        *msg = "collision state: device allocation failed";
        return PICGPU_OOM;
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
        for (int i = 1; i < mc.n_xs; ++i)
            if (!(mc.xs_energy[i] > mc.xs_energy[i - 1])) {
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
        // (sigma v)_max initialisation: FindMaximum (ElectronNeutralCollisionModel.C:383-424)
        double sv = mc.sigma_v_max_init;
        if (!(sv > 0)) {
            const double me = cfg.species[cfg.electron_species].mass;
            const double emax = mc.find_max_energy > 0 ? mc.find_max_energy : xs[mc.n_xs - 1];
            const double step = mc.find_energy_step > 0 ? mc.find_energy_step : emax / 100000.0;
            auto lin = [&](double x, int k) {
                const double* e = xs.data();
                const double* v = xs.data() + size_t(k) * mc.n_xs;
                const int n = mc.n_xs;
                if (x <= e[0]) return v[0];
                if (x >= e[n - 1]) return v[n - 1];
                int lo = 0, hi = n - 1;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) / 2;
                    if (e[mid] <= x) lo = mid; else hi = mid;
                }
                if (e[lo] == x) return v[lo];
                return v[lo] + ((x - e[lo]) / (e[hi] - e[lo])) * (v[hi] - v[lo]);
            };
            sv = 0.0;
            for (double eV = 0.0; eV < emax; eV += step) {
                const double q = lin(eV, 1) + lin(eV, 2) + lin(eV, 3);
                sv = std::fmax(sv, std::sqrt(2.0 * kEch * eV / me) * q);
            }
        }
        std::vector<double> svm(nc, sv), rem(nc);
        // remainders seeded U(0,1) (ElectronNeutralCollisionModel.C:286-296),
        // one Philox stream per cell (host copy of the device generator)
        for (int c = 0; c < nc; ++c) {
            uint32_t key0 = uint32_t(cfg.seed), key1 = uint32_t(cfg.seed >> 32);
            uint32_t x0 = 0, x1 = kStreamRemainder, x2 = uint32_t(c), x3 = 0;
            for (int rr = 0; rr < 10; ++rr) {
                const uint64_t p0 = uint64_t(0xD2511F53u) * x0, p1 = uint64_t(0xCD9E8D57u) * x2;
                const uint32_t n0 = uint32_t(p1 >> 32) ^ x1 ^ key0, n2 = uint32_t(p0 >> 32) ^ x3 ^ key1;
                x1 = uint32_t(p1); x3 = uint32_t(p0); x0 = n0; x2 = n2;
                key0 += 0x9E3779B9u; key1 += 0xBB67AE85u;
            }
            const uint32_t a = x0 >> 5, b = x1 >> 6;
            rem[c] = (double(a) * 67108864.0 + double(b)) * (1.0 / 9007199254740992.0);
        }
        if (dmalloc(&st.svmax, nc) || dmalloc(&st.remainder, nc) || dmalloc(&st.xs, xs.size()) ||
            dmalloc(&st.ncand, nc + 1) || dmalloc(&st.cand_off, nc + 2)) {
            *msg = "MCC state: device allocation failed";
            return PICGPU_OOM;
        }
        cudaMemcpyAsync(st.svmax, svm.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st.remainder, rem.data(), nc * sizeof(double), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st.xs, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            *msg = "MCC state: upload failed";
            return PICGPU_CUDA_ERROR;
        }
    }
    return PICGPU_OK;
}

void collide_free(CollideState& st) {
    void* ptrs[] = {st.svmax, st.remainder, st.xs, st.cell_start, st.cell_count, st.cell_cursor, st.counts,
                    st.scan_tmp, st.ncand, st.cand_off, st.stage, st.flags, st.pos, st.stage_tmp};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int s = 0; s < PICGPU_MAX_SPECIES; ++s) {
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
            order_cells_kernel<<<(nc + 127) / 128, 128, 0, a.stream>>>(nc, start, st.idx[s]);
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
    }
}

}  // namespace

int sort_species(CollideState& st, const DMesh& m, int s, const DSpecies& src, const DSpecies& dst, long n,
                 bool mixed, long* kept, cudaStream_t stream, std::string* msg, int64_t* launches) {
    const int nc = m.n_cells;
    if (!st.cell_start) {
        if (dmalloc(&st.cell_start, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) ||
            dmalloc(&st.cell_count, size_t(PICGPU_MAX_SPECIES) * (nc + 1)) || dmalloc(&st.cell_cursor, nc + 1) ||
            dmalloc(&st.counts, 8) || dmalloc(&st.scan_tmp, (nc + 1) / 1024 + 8)) {
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

int run_collisions(CollideState& st, const CollideArgs& a, int64_t counts[8], long newn[], int swapped[],
                   std::string* msg, int64_t* launches, double* phase_ms) {
    (void)phase_ms;
    const picgpu_config& cfg = *a.cfg;
    const int nc = a.m.n_cells;
    for (int s = 0; s < a.n_species; ++s) { newn[s] = a.n[s]; swapped[s] = 0; }
    cudaMemsetAsync(st.counts, 0, 8 * sizeof(unsigned long long), a.stream);
    // cell occupancy of every species (PICCloud::buildCellOccupancy)
    for (int s = 0; s < a.n_species; ++s) {
        const int e = occupancy(st, a, s, msg, launches);
        if (e) return e;
    }
    // Coulomb first, then electron-neutral (PICCloud::collisions, PICCloud.C:526-539)
    if (cfg.coulomb.enabled) {
        CoulombSpecies C{};
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
        if (a.mixed)
            coulomb_kernel<float><<<(nc + 63) / 64, 64, 0, a.stream>>>(
                C, nc, a.m.vol, cfg.coulomb.coulomb_log, cfg.coulomb.allow_intra, cfg.dt, cfg.seed, uint32_t(a.step),
                st.counts);
        else
            coulomb_kernel<double><<<(nc + 63) / 64, 64, 0, a.stream>>>(
                C, nc, a.m.vol, cfg.coulomb.coulomb_log, cfg.coulomb.allow_intra, cfg.dt, cfg.seed, uint32_t(a.step),
                st.counts);
        *launches += 1;
    }
    if (cfg.mcc.enabled) {
        const picgpu_mcc& mc = cfg.mcc;
        const int es = cfg.electron_species;
        MccParams M{};
        M.n_cells = nc;
        M.e_start = st.cell_start + size_t(es) * (nc + 1);
        M.e_idx = st.idx[es];
        M.svmax = st.svmax;
        M.rem = st.remainder;
        M.xs = st.xs;
        M.n_xs = st.n_xs;
        M.n_gas = mc.gas_density;
        M.mg = mc.gas_mass;
        M.vth_gas = std::sqrt(kKb * mc.gas_temperature / mc.gas_mass);
        M.me = cfg.species[es].mass;
        M.dt = cfg.dt;
        for (int k = 0; k < 3; ++k) M.drift[k] = mc.gas_velocity[k];
        M.ex_th = mc.ex_threshold;
        M.iz_th = mc.iz_threshold;
        M.wEwN = cfg.species[es].weight / mc.gas_weight;
        M.wNwE = 1.0 / M.wEwN;
        M.create_e = mc.create_electron;
        M.create_i = mc.create_ion;
        M.seed = cfg.seed;
        M.step = uint32_t(a.step);
        M.counts = st.counts;
        // candidates per cell and their staging offsets
        mcc_count_kernel<<<(nc + 255) / 256, 256, 0, a.stream>>>(M, st.ncand);
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
        if (a.mixed) mcc_kernel<float><<<(nc + 127) / 128, 128, 0, a.stream>>>(M, a.sp[es], st.stage);
        else mcc_kernel<double><<<(nc + 127) / 128, 128, 0, a.stream>>>(M, a.sp[es], st.stage);
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
    unsigned long long h[8];
    cudaMemcpyAsync(h, st.counts, sizeof h, cudaMemcpyDeviceToHost, a.stream);
    if (cudaStreamSynchronize(a.stream) != cudaSuccess) {
        *msg = "collision step failed";
        return PICGPU_CUDA_ERROR;
    }
    for (int k = 0; k < 8; ++k) counts[k] = (int64_t)h[k];
    return cudaGetLastError() == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

}  // namespace pgd
