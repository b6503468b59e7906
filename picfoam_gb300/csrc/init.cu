// init.cu -- particles created on the device: the InitializationModel
// sub-models of picInitialise (preProcess/picInitialise/InitializationModel)
// and the SimpleInjection boundary model's per-step emission.
//
// Built with --fmad=false: every product and sum rounds on its own, in the
// order of the CPU oracle, which places the same particles bit for bit.
//
//   init_count_kernel        per-tet models: particles per cell; a tet gets
//                            floor(n V / w) plus one with probability equal to
//                            the remainder (EquipartitionInitialization.C:100-117,
//                            MaxwellianInitialization.C:95-110,
//                            IsotropizationInitialization.C:72-90)
//   init_fill_tets_kernel    one warp per cell: the same per-tet counts, then
//                            every particle: a uniform point in its tet, the
//                            empty-axis constraint, U = scale (x) N(0,1)^3 + drift
//   init_fill_cells_kernel   QuasineutralPlasma (QuasineutralPlasmaInitialization.C:102-175):
//                            cellCount parcels per cell in a random tet
//   init_fill_lattice_kernel UniformDisplacement (UniformInitialization.C:51-127):
//                            sinusoidally displaced lattice, located in the mesh
//   inject_kernel            SimpleInjection::injection (SimpleInjection.C:197-240)
//                            through ParticleEmitter::emitParticle
#include "init.h"

#include <algorithm>

namespace pgd {

__constant__ int8_t c_init_tri[12][3];

cudaError_t init_set_tables(const TetConst& t) { return cudaMemcpyToSymbol(c_init_tri, t.tri, sizeof t.tri); }

namespace {

// ----------------------------------------------- deterministic sampling --
// ln x for finite x > 0 in fixed FP64 operations: x = m 2^e with m in
// [sqrt(1/2), sqrt(2)), ln m = 2 atanh(z) with z = (m - 1) / (m + 1),
// |z| <= 0.1716, by the series 2 (z + z^3/3 + ... + z^23/23).
__device__ double det_log(double x) {
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e = e - 1;
    }
    const double z = (m - 1.0) / (m + 1.0);
    const double w = z * z;
    double p = 1.0 / 23.0;
    p = p * w + 1.0 / 21.0;
    p = p * w + 1.0 / 19.0;
    p = p * w + 1.0 / 17.0;
    p = p * w + 1.0 / 15.0;
    p = p * w + 1.0 / 13.0;
    p = p * w + 1.0 / 11.0;
    p = p * w + 1.0 / 9.0;
    p = p * w + 1.0 / 7.0;
    p = p * w + 1.0 / 5.0;
    p = p * w + 1.0 / 3.0;
    const double lm = 2.0 * z + 2.0 * z * (w * p);
    return double(e) * 0.69314718055994530942 + lm;
}

// sin x in fixed FP64 operations for |x| < 1e6: x = k pi + r with pi in two
// parts, |r| <= pi/2, sin x = (-1)^k sin r, sin r by its Taylor series to r^23.
__device__ double det_sin(double x) {
    const double kpi_hi = 3.141592653589793116, kpi_lo = 1.2246467991473532e-16;
    const double k = rint(x / kpi_hi);
    const double r = (x - k * kpi_hi) - k * kpi_lo;
    const double w = r * r;
    double p = -1.0 / 25852016738884976640000.0;  // -1/23!
    p = p * w + 1.0 / 51090942171709440000.0;      // 1/21!
    p = p * w - 1.0 / 121645100408832000.0;        // -1/19!
    p = p * w + 1.0 / 355687428096000.0;           // 1/17!
    p = p * w - 1.0 / 1307674368000.0;             // -1/15!
    p = p * w + 1.0 / 6227020800.0;                // 1/13!
    p = p * w - 1.0 / 39916800.0;                  // -1/11!
    p = p * w + 1.0 / 362880.0;                    // 1/9!
    p = p * w - 1.0 / 5040.0;                      // -1/7!
    p = p * w + 1.0 / 120.0;                       // 1/5!
    p = p * w - 1.0 / 6.0;                         // -1/3!
    const double s = r + r * (w * p);
    const long long ki = (long long)k;
    return (ki & 1) ? -s : s;
}

// e^x in fixed FP64 operations for |x| < 700: x = k ln2 + r with ln 2 in two
// parts, |r| <= ln2 / 2, e^r by its Taylor series to r^17, then 2^k exactly.
__device__ double det_exp(double x) {
    const double ln2_hi = 0.6931471805599452862, ln2_lo = 2.3190468138462996e-17;
    const double k = rint(x / ln2_hi);
    const double r = (x - k * ln2_hi) - k * ln2_lo;
    double p = 1.0 / 355687428096000.0;  // 1/17!
    p = p * r + 1.0 / 20922789888000.0;  // 1/16!
    p = p * r + 1.0 / 1307674368000.0;
    p = p * r + 1.0 / 87178291200.0;
    p = p * r + 1.0 / 6227020800.0;
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return ldexp(p, int(k));
}

// Two standard normal variates by Marsaglia's polar method (rejection of
// points outside the unit disc; at most 64 tries, then zeros).
__device__ void polar_pair(Philox& r, double& n1, double& n2) {
    for (int a = 0; a < 64; ++a) {
        const double u1 = 2.0 * r.uniform() - 1.0;
        const double u2 = 2.0 * r.uniform() - 1.0;
        const double s = u1 * u1 + u2 * u2;
        if (s > 0.0 && s < 1.0) {
            const double f = sqrt(-2.0 * det_log(s) / s);
            n1 = u1 * f;
            n2 = u2 * f;
            return;
        }
    }
    n1 = 0.0;
    n2 = 0.0;
}

// sampleNormal<vector>: three variates, components in order.
__device__ void normal3(Philox& r, double* n) {
    double a, b;
    polar_pair(r, a, b);
    n[0] = a;
    n[1] = b;
    polar_pair(r, a, b);
    n[2] = a;
}

// Uniform point in a tet (tetPointRef::randomPoint) by folding the unit cube
// (Rocchini & Cignoni 2000); y gets the coordinates of the three face points
// (the cell-centre coordinate is 1 - y0 - y1 - y2).
__device__ void tet_point(Philox& r, double* y) {
    double s = r.uniform();
    double t = r.uniform();
    double u = r.uniform();
    if (s + t > 1.0) {
        s = 1.0 - s;
        t = 1.0 - t;
    }
    if (t + u > 1.0) {
        const double tmp = u;
        u = 1.0 - s - t;
        t = 1.0 - tmp;
    } else if (s + t + u > 1.0) {
        const double tmp = u;
        u = s + t + u - 1.0;
        s = 1.0 - t - tmp;
    }
    y[0] = s;
    y[1] = t;
    y[2] = u;
}

// Tet of cell c containing x (the one whose smallest barycentric coordinate
// is largest), coordinates clamped to >= 0 and renormalised.  False when x is
// outside the cell by more than 1e-9.
__device__ bool locate_in_cell(const DMesh& m, int c, const double* x, int& tet, double* y) {
    const int cls = m.cell_class[c];
    double r[3];
    for (int a = 0; a < 3; ++a) r[a] = x[a] - m.cc[3 * size_t(c) + a];
    int best = -1;
    double best_min = -1e300, by[3] = {0, 0, 0};
    for (int t = 0; t < 12; ++t) {
        const double* inv = m.tetinv + (size_t(cls) * 12 + t) * 9;
        double q[3];
        for (int a = 0; a < 3; ++a) q[a] = inv[3 * a] * r[0] + inv[3 * a + 1] * r[1] + inv[3 * a + 2] * r[2];
        const double q0 = 1.0 - q[0] - q[1] - q[2];
        const double mn = fmin(fmin(q0, q[0]), fmin(q[1], q[2]));
        if (mn > best_min) {
            best_min = mn;
            best = t;
            by[0] = q[0];
            by[1] = q[1];
            by[2] = q[2];
        }
    }
    if (best_min < -1e-9) return false;
    const double y0 = 1.0 - by[0] - by[1] - by[2];
    const double yy[4] = {fmax(y0, 0.0), fmax(by[0], 0.0), fmax(by[1], 0.0), fmax(by[2], 0.0)};
    const double s = yy[0] + yy[1] + yy[2] + yy[3];
    for (int a = 0; a < 3; ++a) y[a] = yy[a + 1] / s;
    tet = best;
    return true;
}

// meshTools::constrainDirection applied to the point: its components along
// the empty axes are set to zero, then the point is located again in its cell.
__device__ bool constrain(const InitParams& P, int c, int& t, double* y) {
    const DMesh& m = P.m;
    const double* off = m.offset + size_t(m.cell_class[c]) * 24;
    double x[3];
    for (int a = 0; a < 3; ++a)
        x[a] = m.cc[3 * size_t(c) + a] + y[0] * off[3 * c_init_tri[t][0] + a] + y[1] * off[3 * c_init_tri[t][1] + a] +
               y[2] * off[3 * c_init_tri[t][2] + a];
    for (int a = 0; a < 3; ++a)
        if (m.empty[a]) x[a] = 0.0;
    return locate_in_cell(m, c, x, t, y);
}

__device__ void store(const InitParams& P, long long i, int tet, const double* y, const double* U) {
    P.tet[i] = tet;
    if (P.y64[0]) {
        for (int a = 0; a < 3; ++a) {
            P.y64[a][i] = y[a];
            P.u64[a][i] = U[a];
        }
    } else {
        for (int a = 0; a < 3; ++a) {
            P.y32[a][i] = float(y[a]);
            P.u32[a][i] = float(U[a]);
        }
    }
}

__device__ void store_inject(const InjectParams& P, long long i, int tet, const double* y, const double* U) {
    P.tet[i] = tet;
    if (P.y64[0]) {
        for (int a = 0; a < 3; ++a) {
            P.y64[a][i] = y[a];
            P.u64[a][i] = U[a];
        }
    } else {
        for (int a = 0; a < 3; ++a) {
            P.y32[a][i] = float(y[a]);
            P.u32[a][i] = float(U[a]);
        }
    }
}

__device__ void velocity(const InitParams& P, Philox& r, double* U) {
    double n[3];
    normal3(r, n);
    for (int a = 0; a < 3; ++a) U[a] = P.sp.scale[a] * n[a] + P.sp.drift[a];
}

// particlesRequired = n V / w; floor, plus one when the remainder exceeds a
// uniform draw of the tet's own stream.
__device__ int tet_count(const InitParams& P, int c, int t, double V) {
    const double req = (P.sp.n * V) / P.sp.w;
    long long k = (long long)req;
    Philox r(P.seed, kStreamInitCount | uint32_t(P.species), uint32_t(c), uint32_t(t));
    if (req - double(k) > r.uniform()) ++k;
    if (k >= (1LL << 24)) {
        *P.error = 2;
        k = 0;
    }
    return int(k);
}

__global__ void __launch_bounds__(256) init_count_kernel(InitParams P, int* counts) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.m.n_cells) return;
    const double* V = P.tet_vol + 12 * size_t(P.m.cell_class[c]);
    int total = 0;
    for (int t = 0; t < 12; ++t) total += tet_count(P, c, t, V[t]);
    counts[c] = total;
}

// One warp per cell; particle j of the cell lies in the tet whose running
// count first exceeds j and is particle k = j - (count before that tet) of it.
__global__ void __launch_bounds__(256) init_fill_tets_kernel(InitParams P, const long long* offsets) {
    const int c = int((long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= P.m.n_cells) return;
    const double* V = P.tet_vol + 12 * size_t(P.m.cell_class[c]);
    const int cnt = lane < 12 ? tet_count(P, c, lane, V[lane]) : 0;
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    int incs[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) incs[q] = __shfl_sync(0xffffffffu, inc, q);
    const int total = incs[11];
    const long long base = P.first + offsets[c];
    for (int j = lane; j < total; j += 32) {
        int t = 0;
        while (t < 11 && incs[t] <= j) ++t;
        const int k = j - (t > 0 ? incs[t - 1] : 0);
        Philox r(P.seed, kStreamInitParticle | uint32_t(P.species), uint32_t(c), (uint32_t(t) << 24) | uint32_t(k));
        double y[3], U[3];
        tet_point(r, y);
        int tt = t;
        if (P.constrain && !constrain(P, c, tt, y)) *P.error = 1;
        velocity(P, r, U);
        store(P, base + j, 12 * c + tt, y, U);
    }
}

__global__ void __launch_bounds__(256) init_fill_cells_kernel(InitParams P) {
    const long long cc = P.sp.cell_count;
    const long long total = cc * P.m.n_cells;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = int(i / cc);
        const long long k = i - cc * c;
        Philox r(P.seed, kStreamInitParticle | uint32_t(P.species), uint32_t(c), uint32_t(k));
        // label((cellTets.size() - 1.0) * scalar01()): tets 0..10 (the last
        // tet of a cell is never chosen, as in picFoam)
        const int t0 = int((12.0 - 1.0) * r.uniform());
        double y[3], U[3];
        tet_point(r, y);
        int tt = t0;
        if (P.constrain && !constrain(P, c, tt, y)) *P.error = 1;
        if (P.use_maxwellian) {
            velocity(P, r, U);
        } else {
            // sample01<vector> normalised: a direction in the positive octant
            double d[3];
            d[0] = r.uniform();
            d[1] = r.uniform();
            d[2] = r.uniform();
            const double inv = 1.0 / sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            for (int a = 0; a < 3; ++a) U[a] = (d[a] * inv) * P.sp.speed;
        }
        store(P, P.first + i, 12 * c + tt, y, U);
    }
}

__global__ void __launch_bounds__(256) init_fill_lattice_kernel(InitParams P) {
    const long long ny = P.nl[1], nz = P.nl[2];
    const long long total = P.nl[0] * ny * nz;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long i = idx / (ny * nz);
        const long long j = (idx / nz) % ny;
        const long long k = idx % nz;
        const double p[3] = {P.lo[0] + P.delta[0] * double(i), P.lo[1] + P.delta[1] * double(j),
                             P.lo[2] + P.delta[2] * double(k)};
        const double dist = (p[0] - P.lo[0]) * P.dir[0] + (p[1] - P.lo[1]) * P.dir[1] + (p[2] - P.lo[2]) * P.dir[2];
        const double cur = P.sp.displacement * det_sin(dist / P.span_len * P.cycles * 3.141592653589793116);
        double x[3];
        for (int a = 0; a < 3; ++a) x[a] = p[a] + P.dir[a] * cur;
        // the block cell holding x, then the tet
        int ijk[3];
        bool inside = true;
        for (int a = 0; a < 3; ++a) {
            const double s = (x[a] - P.grid_lo[a]) / (P.grid_hi[a] - P.grid_lo[a]) * P.grid_n[a];
            int q = 0;
            if (s >= -1e-9 && s <= P.grid_n[a] + 1e-9) {
                q = int(floor(s));
                q = q < 0 ? 0 : (q >= P.grid_n[a] ? P.grid_n[a] - 1 : q);
            } else {
                inside = false;
            }
            ijk[a] = q;
        }
        int c = -1, t = 0;
        double y[3] = {0, 0, 0};
        if (inside) c = P.grid_cell[ijk[0] + size_t(P.grid_n[0]) * (ijk[1] + size_t(P.grid_n[1]) * ijk[2])];
        if (c < 0 || !locate_in_cell(P.m, c, x, t, y)) {
            *P.error = 1;
            c = 0;
            t = 0;
            y[0] = y[1] = y[2] = 0.0;
        }
        Philox r(P.seed, kStreamInitLattice | uint32_t(P.species), uint32_t(idx >> 32), uint32_t(idx));
        double U[3];
        velocity(P, r, U);
        store(P, P.first + idx, 12 * c + t, y, U);
    }
}

__global__ void __launch_bounds__(256) init_occupancy_kernel(const int32_t* __restrict__ tet, long long n,
                                                             int* counts) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int t = tet[i];
        if (t >= 0) atomicAdd(counts + t / 12, 1);
    }
}

__global__ void __launch_bounds__(1024) init_minmax_kernel(const int* __restrict__ counts, int n, long long* out) {
    __shared__ long long smin[1024], smax[1024], ssum[1024];
    long long mn = n > 0 ? (1LL << 62) : 0, mx = 0, sm = 0;
    for (int i = threadIdx.x; i < n; i += 1024) {
        const long long v = counts[i];
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
        sm += v;
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int o = 512; o >= 1; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = min(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = max(smax[threadIdx.x], smax[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = smin[0];
        out[1] = smax[0];
        out[2] = ssum[0];
    }
}

// ------------------------------------------------------------ injection --
// ParticleEmitter::emitParticle (ParticleEmitter.C:265-418): area-weighted
// triangle, uniform point on it (Osada, Funkhouser, Chazelle & Dobkin 2002:
// (1 - sqrt r1) A + sqrt r1 (1 - r2) B + sqrt r1 r2 C), moved a = U(0.1, 0.5)
// of the normal distance towards the cell centre, velocity about the inward
// normal n with tangents t1 = (face centre - first triangle point) / |.|,
// t2 = n x t1 / |.|, the empty-axis constraint, located in the owner cell.
__global__ void __launch_bounds__(256) inject_kernel(InjectParams P) {
    const double kB = 1.380649e-23;
    if (blockIdx.x == 0 && threadIdx.x == 0 && P.qconv) P.qconv[P.patch] = P.qconv[P.patch] - P.ejected_charge;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < P.n;
         k += (long long)gridDim.x * blockDim.x) {
        Philox r(P.seed, kStreamInject | (uint32_t(P.injector) << 4) | uint32_t(P.species), P.step, uint32_t(k));
        const double af = r.uniform() * P.area;
        // the largest i with af > cum[i] (cum[0] = 0): the triangle holding af
        int lo = 0, hi = P.n_tri - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (af > P.tri_cum[mid]) lo = mid;
            else hi = mid - 1;
        }
        const int tri = lo;
        const int c = P.tri_cell[tri], t = P.tri_tet[tri];
        const double* off = P.m.offset + size_t(P.m.cell_class[c]) * 24;
        const double* cc = P.m.cc + 3 * size_t(c);
        double A[3], B[3], C[3];
        for (int a = 0; a < 3; ++a) {
            A[a] = cc[a] + off[3 * c_init_tri[t][0] + a];
            B[a] = cc[a] + off[3 * c_init_tri[t][1] + a];
            C[a] = cc[a] + off[3 * c_init_tri[t][2] + a];
        }
        const double r1 = r.uniform(), r2 = r.uniform();
        const double sr = sqrt(r1);
        double pf[3];
        for (int a = 0; a < 3; ++a) pf[a] = (1.0 - sr) * A[a] + sr * (1.0 - r2) * B[a] + sr * r2 * C[a];
        const double fa = 0.1 + 0.4 * r.uniform();
        const double* nrm = P.tri_normal + 3 * size_t(tri);
        const double dn = fabs((pf[0] - cc[0]) * nrm[0] + (pf[1] - cc[1]) * nrm[1] + (pf[2] - cc[2]) * nrm[2]);
        double x[3];
        for (int a = 0; a < 3; ++a) x[a] = pf[a] - fa * (dn * nrm[a]);
        // tangents and the inward normal
        const double* fc = P.tri_fc + 3 * size_t(tri);
        double n[3], t1[3], t2[3];
        for (int a = 0; a < 3; ++a) {
            n[a] = -nrm[a];
            t1[a] = fc[a] - A[a];
        }
        const double m1 = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        for (int a = 0; a < 3; ++a) t1[a] = t1[a] / m1;
        t2[0] = n[1] * t1[2] - n[2] * t1[1];
        t2[1] = n[2] * t1[0] - n[0] * t1[2];
        t2[2] = n[0] * t1[1] - n[1] * t1[0];
        const double m2 = sqrt(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]);
        for (int a = 0; a < 3; ++a) t2[a] = t2[a] / m2;
        // velocity models (ParticleEmitter.C:420-535)
        double U[3];
        const double vt = sqrt(kB * P.temperature / P.mass);
        if (P.model == PICGPU_EMIT_MOST_PROBABLE_SPEED) {
            const double vmp = sqrt(2.0 * kB * P.temperature / P.mass);
            for (int a = 0; a < 3; ++a) U[a] = vmp * n[a];
        } else {
            double n1, n2;
            polar_pair(r, n1, n2);
            double tg[3];
            for (int a = 0; a < 3; ++a) tg[a] = vt * (n1 * t1[a] + n2 * t2[a]);
            double un;
            if (P.model == PICGPU_EMIT_BIRD_MAXWELLIAN_FLUX) {
                const double vmp = sqrt(2.0 * kB * P.temperature / P.mass);
                double u = 0.0;
                for (int it = 0; it < 1000; ++it) {
                    u = 3.0 * (2.0 * r.uniform() - 1.0);
                    const double pr = u < 0.0 ? -1.0 : 2.0 * u / 1.4142135623730951 * det_exp(0.5 - u * u);
                    if (!(pr < r.uniform())) break;
                }
                un = vmp * u;
            } else if (P.model == PICGPU_EMIT_HALF_MAXWELLIAN_FLUX) {
                double n3, n4;
                polar_pair(r, n3, n4);
                un = fabs(n3) * vt;
            } else {  // maxwellianFlux
                const double R = r.uniform();
                un = vt * sqrt(-2.0 * det_log(1.0 - R));
            }
            for (int a = 0; a < 3; ++a) U[a] = tg[a] + un * n[a];
        }
        for (int a = 0; a < 3; ++a)
            if (P.constrain && P.m.empty[a]) x[a] = 0.0;
        int tt = 0;
        double y[3] = {0, 0, 0};
        if (!locate_in_cell(P.m, c, x, tt, y)) *P.error = 1;
        store_inject(P, P.first + k, 12 * c + tt, y, U);
    }
}

// FreeStream::injection (FreeStream.C:126-396): the face accumulator gains
// its share of the flux; the integer part is emitted, plus one parcel when
// the remainder exceeds a uniform draw.
__global__ void __launch_bounds__(256) freestream_count_kernel(FreeStreamParams P) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < P.n_faces; f += gridDim.x * blockDim.x) {
        const size_t i = size_t(f) * P.n_species + P.j;
        double a = P.acc[i] + P.add[i];
        long long n = a < 2.0e9 ? (long long)a : (1LL << 31);
        if (n < 0) n = 0;
        Philox r(P.seed, kStreamFreeStreamCount | (uint32_t(P.injector) << 4) | uint32_t(P.species), P.step,
                 uint32_t(f));
        if (a - double(n) > r.uniform()) ++n;
        if (n > (1LL << 30)) {
            *P.error = 2;
            n = 0;
        }
        P.acc[i] = a - double(n);
        P.counts[f] = int(n);
    }
}

// The parcels of one face: a face triangle by area share, a uniform point on
// it (barycentric 0 at the cell centre), the normal speed ratio by Bird's
// acceptance-rejection (eq. 12.5, the QA scaling of DSMC3), thermal
// tangential components and the drift's tangential part.
__global__ void __launch_bounds__(256) freestream_emit_kernel(FreeStreamParams P) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < P.n_faces; f += gridDim.x * blockDim.x) {
        const int cnt = P.counts[f];
        if (cnt == 0) continue;
        Philox r(P.seed, kStreamFreeStream | (uint32_t(P.injector) << 4) | uint32_t(P.species), P.step,
                 uint32_t(f));
        const double s = P.s[size_t(f) * P.n_species + P.j];
        const double root = sqrt(s * s + 2.0);
        const double qa = s + root;
        const double qb = 0.5 * (1.0 + s * (s - root));
        const double scaling = s < -3.0 ? fabs(s) + 1.0 : 3.0;
        const double* n = P.n_in + 3 * size_t(f);
        const double* t1 = P.t1 + 3 * size_t(f);
        const double* t2 = P.t2 + 3 * size_t(f);
        const double d1 = t1[0] * P.U[0] + t1[1] * P.U[1] + t1[2] * P.U[2];
        const double d2 = t2[0] * P.U[0] + t2[1] * P.U[1] + t2[2] * P.U[2];
        const int c = P.cell[f];
        const long long base = P.first + P.offsets[f];
        for (int k = 0; k < cnt; ++k) {
            const double sel = r.uniform();
            const int t = P.tet0[f] + (P.frac0[f] >= sel ? 0 : 1);
            const double r1 = r.uniform(), r2 = r.uniform();
            const double sr = sqrt(r1);
            const double y[3] = {1.0 - sr, sr * (1.0 - r2), sr * r2};
            double u = 0.0;
            for (int it = 0; it < 10000; ++it) {
                const double ut = scaling * (2.0 * r.uniform() - 1.0);
                u = ut + s;
                const double pr = u < 0.0 ? -1.0 : 2.0 * u / qa * det_exp(qb - ut * ut);
                if (!(pr < r.uniform())) break;
            }
            double n1, n2;
            polar_pair(r, n1, n2);
            double U[3];
            for (int a = 0; a < 3; ++a)
                U[a] = ((P.v_t * (n1 * t1[a] + n2 * t2[a]) + d1 * t1[a]) + d2 * t2[a]) + P.c_mp * u * n[a];
            const long long i = base + k;
            P.tet[i] = 12 * c + t;
            if (P.y64[0]) {
                for (int a = 0; a < 3; ++a) {
                    P.y64[a][i] = y[a];
                    P.u64[a][i] = U[a];
                }
            } else {
                for (int a = 0; a < 3; ++a) {
                    P.y32[a][i] = float(y[a]);
                    P.u32[a][i] = float(U[a]);
                }
            }
        }
    }
}

// ------------------------------------------------------------- scan ------
constexpr int kScanChunk = 1024;  // 256 threads x 4 counts

__global__ void __launch_bounds__(256) scan_sums_kernel(const int* __restrict__ counts, int n, long long* sums) {
    __shared__ long long ws[256];
    const long long base = (long long)blockIdx.x * kScanChunk + 4 * threadIdx.x;
    long long s = 0;
    for (int q = 0; q < 4; ++q)
        if (base + q < n) s += counts[base + q];
    ws[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o >= 1; o >>= 1) {
        if (threadIdx.x < o) ws[threadIdx.x] += ws[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = ws[0];
}

// Exclusive scan of the block sums in place, by one block in chunks of 1024.
__global__ void __launch_bounds__(1024) scan_block_sums_kernel(long long* sums, int nb) {
    __shared__ long long ws[1024];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += 1024) {
        const int i = b0 + threadIdx.x;
        const long long v = i < nb ? sums[i] : 0;
        ws[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const long long y = threadIdx.x >= o ? ws[threadIdx.x - o] : 0;
            __syncthreads();
            ws[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + ws[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += ws[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void __launch_bounds__(256) scan_apply_kernel(const int* __restrict__ counts, int n,
                                                         const long long* __restrict__ sums, long long* offsets) {
    __shared__ long long ws[256];
    const long long base = (long long)blockIdx.x * kScanChunk + 4 * threadIdx.x;
    long long v[4], s = 0;
    for (int q = 0; q < 4; ++q) {
        v[q] = base + q < n ? counts[base + q] : 0;
        s += v[q];
    }
    ws[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const long long y = threadIdx.x >= o ? ws[threadIdx.x - o] : 0;
        __syncthreads();
        ws[threadIdx.x] += y;
        __syncthreads();
    }
    long long run = sums[blockIdx.x] + ws[threadIdx.x] - s;
    for (int q = 0; q < 4; ++q) {
        if (base + q < n) offsets[base + q] = run;
        run += v[q];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) offsets[n] = sums[gridDim.x];
}

inline int nblocks(long long n, int bs, int cap) { return int(std::min<long long>((n + bs - 1) / bs, cap)); }

}  // namespace

void launch_init_count(const InitParams& P, int* counts, cudaStream_t s) {
    init_count_kernel<<<nblocks(P.m.n_cells, 256, 1 << 30), 256, 0, s>>>(P, counts);
}

void launch_freestream_count(const FreeStreamParams& P, cudaStream_t s) {
    if (P.n_faces > 0) freestream_count_kernel<<<nblocks(P.n_faces, 256, 152 * 16), 256, 0, s>>>(P);
}

void launch_freestream_emit(const FreeStreamParams& P, cudaStream_t s) {
    if (P.n_faces > 0) freestream_emit_kernel<<<nblocks(P.n_faces, 256, 152 * 16), 256, 0, s>>>(P);
}

long long init_scan_scratch(int n) { return (n + kScanChunk - 1) / kScanChunk + 1; }

cudaError_t init_scan(const int* counts, long long* offsets, long long* block_sums, int n, cudaStream_t s) {
    const int nb = int((n + kScanChunk - 1) / kScanChunk);
    if (nb == 0) return cudaMemsetAsync(offsets, 0, sizeof(long long), s);
    scan_sums_kernel<<<nb, 256, 0, s>>>(counts, n, block_sums);
    scan_block_sums_kernel<<<1, 1024, 0, s>>>(block_sums, nb);
    scan_apply_kernel<<<nb, 256, 0, s>>>(counts, n, block_sums, offsets);
    return cudaGetLastError();
}

void launch_init_fill_tets(const InitParams& P, const long long* offsets, cudaStream_t s) {
    init_fill_tets_kernel<<<nblocks(32LL * P.m.n_cells, 256, 1 << 30), 256, 0, s>>>(P, offsets);
}

void launch_init_fill_cells(const InitParams& P, cudaStream_t s) {
    const long long total = (long long)P.sp.cell_count * P.m.n_cells;
    if (total > 0) init_fill_cells_kernel<<<nblocks(total, 256, 152 * 64), 256, 0, s>>>(P);
}

void launch_init_fill_lattice(const InitParams& P, cudaStream_t s) {
    const long long total = P.nl[0] * P.nl[1] * P.nl[2];
    if (total > 0) init_fill_lattice_kernel<<<nblocks(total, 256, 152 * 64), 256, 0, s>>>(P);
}

void launch_init_occupancy(const int32_t* tet, long long n, int n_cells, int* counts, cudaStream_t s) {
    cudaMemsetAsync(counts, 0, size_t(n_cells) * sizeof(int), s);
    if (n > 0) init_occupancy_kernel<<<nblocks(n, 256, 152 * 64), 256, 0, s>>>(tet, n, counts);
}

void launch_inject(const InjectParams& P, cudaStream_t s) {
    if (P.n > 0 || P.qconv) inject_kernel<<<std::max(1, nblocks(P.n, 256, 152 * 32)), 256, 0, s>>>(P);
}

void launch_init_minmax(const int* counts, int n, long long* out, cudaStream_t s) {
    init_minmax_kernel<<<1, 1024, 0, s>>>(counts, n, out);
}

}  // namespace pgd
