// particles.cu -- particle store maintenance: stable removal of absorbed
// particles (the parcels Cloud::move deletes when keepParticle is false,
// PICParcel.C:70) from the structure-of-arrays store.
#include "particles.h"

#include <algorithm>

namespace pgd {

namespace {

constexpr int kItems = 4;
constexpr int kBlock = 256;
constexpr int kTile = kItems * kBlock;  // 1024 particles per block

__global__ void count_alive_kernel(const int32_t* __restrict__ tet, long n, int* __restrict__ counts) {
    __shared__ int ws[kBlock / 32];
    const long base = long(blockIdx.x) * kTile + long(threadIdx.x) * kItems;
    int c = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
        if (base + k < n && tet[base + k] >= 0) ++c;
    for (int off = 16; off >= 1; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kBlock / 32; ++w) t += ws[w];
        counts[blockIdx.x] = t;
    }
}

// Exclusive scan of counts[0..n) in place; counts[n] receives the total.
__global__ void scan_single_kernel(int* counts, long n) {
    __shared__ int ws[32];
    __shared__ long long carry_s;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (long base = 0; base < n; base += blockDim.x) {
        const long i = base + threadIdx.x;
        const int v = i < n ? counts[i] : 0;
        int x = v;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = lane < int(blockDim.x >> 5) ? ws[lane] : 0;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            ws[lane] = w;
        }
        __syncthreads();
        const int incl = x + (warp > 0 ? ws[warp - 1] : 0);
        const long long carry = carry_s;
        if (i < n) counts[i] = int(carry + incl - v);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry_s = carry + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[n] = int(carry_s);
}

template <class R>
__global__ void scatter_kernel(const int32_t* __restrict__ tet, const R* __restrict__ y0,
                               const R* __restrict__ y1, const R* __restrict__ y2, const R* __restrict__ u0,
                               const R* __restrict__ u1, const R* __restrict__ u2, int32_t* __restrict__ otet,
                               R* __restrict__ oy0, R* __restrict__ oy1, R* __restrict__ oy2,
                               R* __restrict__ ou0, R* __restrict__ ou1, R* __restrict__ ou2, long n,
                               const int* __restrict__ offsets, const double* __restrict__ nw,
                               const int32_t* __restrict__ zq, double* __restrict__ onw,
                               int32_t* __restrict__ ozq) {
    __shared__ int ws[kBlock / 32];
    const long base = long(blockIdx.x) * kTile + long(threadIdx.x) * kItems;
    bool f[kItems];
    int c = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        f[k] = base + k < n && tet[base + k] >= 0;
        c += f[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = c;
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    int woff = 0;
    for (int w = 0; w < warp; ++w) woff += ws[w];
    long pos = long(offsets[blockIdx.x]) + woff + x - c;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        if (!f[k]) continue;
        const long i = base + k;
        otet[pos] = tet[i];
        oy0[pos] = y0[i]; oy1[pos] = y1[i]; oy2[pos] = y2[i];
        ou0[pos] = u0[i]; ou1[pos] = u1[i]; ou2[pos] = u2[i];
        if (nw) {
            onw[pos] = nw[i];
            ozq[pos] = zq[i];
        }
        ++pos;
    }
}

}  // namespace

long compact_blocks(long n) { return (n + kTile - 1) / kTile; }

namespace {

// Host row-major arrays (n x 3 FP64) <-> the structure-of-arrays store.
__global__ void check_tets_kernel(const int32_t* __restrict__ tet, long n, long long ntet, int* bad) {
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        if (tet[i] < 0 || tet[i] >= ntet) *bad = 1;
}

template <class Real>
__global__ void scatter_rows_kernel(const int32_t* __restrict__ tet, const double* __restrict__ bary,
                                    const double* __restrict__ U, long n, DSpecies dst) {
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        dst.tet[i] = tet[i];
        for (int a = 0; a < 3; ++a) {
            if (sizeof(Real) == 8) {
                dst.y64[a][i] = bary[3 * i + a];
                dst.u64[a][i] = U[3 * i + a];
            } else {
                dst.y32[a][i] = float(bary[3 * i + a]);
                dst.u32[a][i] = float(U[3 * i + a]);
            }
        }
    }
}

template <class Real>
__global__ void gather_rows_kernel(DSpecies src, long n, int32_t* __restrict__ tet, double* __restrict__ bary,
                                   double* __restrict__ U) {
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        tet[i] = src.tet[i];
        for (int a = 0; a < 3; ++a) {
            if (sizeof(Real) == 8) {
                bary[3 * i + a] = src.y64[a][i];
                U[3 * i + a] = src.u64[a][i];
            } else {
                bary[3 * i + a] = double(src.y32[a][i]);
                U[3 * i + a] = double(src.u32[a][i]);
            }
        }
    }
}

__global__ void fill_attributes_kernel(double* __restrict__ nw, int32_t* __restrict__ zq, long from, long to,
                                       double weight) {
    for (long i = from + blockIdx.x * long(blockDim.x) + threadIdx.x; i < to; i += long(gridDim.x) * blockDim.x) {
        nw[i] = weight;
        zq[i] = 1;
    }
}

}  // namespace

void launch_fill_attributes(const DSpecies& d, long from, long to, double weight, cudaStream_t s) {
    if (!d.nw || to <= from) return;
    const int g = int(std::min<long>((to - from + 255) / 256, 152 * 16));
    fill_attributes_kernel<<<g, 256, 0, s>>>(d.nw, d.zq, from, to, weight);
}

void launch_check_tets(const int32_t* tet, long n, long long ntet, int* bad, cudaStream_t s) {
    if (n > 0) check_tets_kernel<<<int(std::min<long>((n + 255) / 256, 152 * 16)), 256, 0, s>>>(tet, n, ntet, bad);
}

void launch_scatter_rows(const int32_t* tet, const double* bary, const double* U, long n, const DSpecies& dst,
                         bool fp32, cudaStream_t s) {
    if (n <= 0) return;
    const int g = int(std::min<long>((n + 255) / 256, 152 * 16));
    if (fp32) scatter_rows_kernel<float><<<g, 256, 0, s>>>(tet, bary, U, n, dst);
    else scatter_rows_kernel<double><<<g, 256, 0, s>>>(tet, bary, U, n, dst);
}

void launch_gather_rows(const DSpecies& src, long n, bool fp32, int32_t* tet, double* bary, double* U,
                        cudaStream_t s) {
    if (n <= 0) return;
    const int g = int(std::min<long>((n + 255) / 256, 152 * 16));
    if (fp32) gather_rows_kernel<float><<<g, 256, 0, s>>>(src, n, tet, bary, U);
    else gather_rows_kernel<double><<<g, 256, 0, s>>>(src, n, tet, bary, U);
}

cudaError_t compact_species(const DSpecies& src, const DSpecies& dst, long n, bool mixed, int* scan,
                            long* kept, cudaStream_t s) {
    const long nblk = compact_blocks(n);
    if (nblk == 0) { *kept = 0; return cudaSuccess; }
    count_alive_kernel<<<unsigned(nblk), kBlock, 0, s>>>(src.tet, n, scan);
    scan_single_kernel<<<1, 1024, 0, s>>>(scan, nblk);
    if (mixed)
        scatter_kernel<float><<<unsigned(nblk), kBlock, 0, s>>>(
            src.tet, src.y32[0], src.y32[1], src.y32[2], src.u32[0], src.u32[1], src.u32[2], dst.tet, dst.y32[0],
            dst.y32[1], dst.y32[2], dst.u32[0], dst.u32[1], dst.u32[2], n, scan, src.nw, src.zq, dst.nw, dst.zq);
    else
        scatter_kernel<double><<<unsigned(nblk), kBlock, 0, s>>>(
            src.tet, src.y64[0], src.y64[1], src.y64[2], src.u64[0], src.u64[1], src.u64[2], dst.tet, dst.y64[0],
            dst.y64[1], dst.y64[2], dst.u64[0], dst.u64[1], dst.u64[2], n, scan, src.nw, src.zq, dst.nw, dst.zq);
    int total = 0;
    cudaError_t e = cudaMemcpyAsync(&total, scan + nblk, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    *kept = total;
    return cudaGetLastError();
}

}  // namespace pgd
