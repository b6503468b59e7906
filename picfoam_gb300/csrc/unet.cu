// unet.cu -- the U-Net of the learned Poisson warm start: layers, forward,
// backward and Adam on the GPU.
//
// Architecture (3 levels, 16/32/64 channels, 3x3x3 convolutions, no biases,
// so the net is positively homogeneous: net(k x) = k net(x) for k > 0):
//
//   in [V][2] (scaled residual, domain mask)
//   a1  = relu(c1a(in))            2 -> 16   CUDA cores (FP32)
//   a2  = relu(c1b(a1))           16 -> 16   tensor cores
//   a3  = relu(c2a(pool(a2)))     16 -> 32   (V/8)
//   a4  = relu(c2b(a3))           32 -> 32
//   a5  = relu(c3a(pool(a4)))     32 -> 64   (V/64)
//   a6  = relu(c3b(a5))           64 -> 64
//   a7  = relu(d2a([up(a6), a4])) 96 -> 32   (V/8)
//   a8  = relu(d2b(a7))           32 -> 32
//   a9  = relu(d1a([up(a8), a2])) 48 -> 16   (V)
//   a10 = relu(d1b(a9))           16 -> 16
//   out = co(a10)                 16 -> 1    CUDA cores (FP32)
//
// Activations are BF16 channels-last; tensor-core layers take BF16 weights
// packed from the FP32 master copy, accumulate in FP32.  Backward: the input
// gradient of a tensor-core layer is the same tensor-core convolution with
// the flipped, transposed weights (FP32 out); weight gradients accumulate in
// FP32 on the CUDA cores.  Pooling is a 2x2x2 average, upsampling nearest.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "unet_net.h"

namespace pgd {

const UNetLayerDef kUNetLayers[kUNetNumLayers] = {
    {2, 16}, {16, 16}, {16, 32}, {32, 32}, {32, 64}, {64, 64}, {96, 32}, {32, 32}, {48, 16}, {16, 16}, {16, 1}};

namespace {

__device__ __forceinline__ float bf(__nv_bfloat16 h) { return __bfloat162float(h); }

__device__ __forceinline__ void load8(const __nv_bfloat16* p, float* f) {
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}

__device__ __forceinline__ void store16_bf16(__nv_bfloat16* p, const float* f) {
    __nv_bfloat162 h[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    uint4* o = reinterpret_cast<uint4*>(p);
    o[0] = *reinterpret_cast<uint4*>(&h[0]);
    o[1] = *reinterpret_cast<uint4*>(&h[4]);
}

struct Coord {
    int x, y, z;
};

__device__ __forceinline__ Coord coord(long v, const ConvGrid& g) {
    return {int(v % g.X), int((v / g.X) % g.Y), int(v / (long(g.X) * g.Y))};
}

__device__ __forceinline__ bool neighbour(const Coord& c, int t, const ConvGrid& g, int sign, long* nv) {
    const int dz = (t / 9 - 1) * sign, dy = ((t / 3) % 3 - 1) * sign, dx = (t % 3 - 1) * sign;
    const int xn = c.x + dx, yn = c.y + dy, zn = c.z + dz;
    if (xn < 0 || xn >= g.X || yn < 0 || yn >= g.Y || zn < 0 || zn >= g.Z) return false;
    *nv = (long(zn) * g.Y + yn) * g.X + xn;
    return true;
}

// a1 = relu(conv(in, w)), in FP32 [V][2], w FP32 [27][16][2].
__global__ void conv_first_kernel(ConvGrid g, const float* __restrict__ in, const float* __restrict__ w,
                                  __nv_bfloat16* __restrict__ out) {
    __shared__ float ws[27 * 16 * 2];
    for (int i = threadIdx.x; i < 27 * 16 * 2; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    const long V = long(g.X) * g.Y * g.Z;
    const long v = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const Coord c = coord(v, g);
    float acc[16];
#pragma unroll
    for (int o = 0; o < 16; ++o) acc[o] = 0.f;
    for (int t = 0; t < 27; ++t) {
        long nv;
        if (!neighbour(c, t, g, 1, &nv)) continue;
        const float2 i2 = __ldg(reinterpret_cast<const float2*>(in) + nv);
#pragma unroll
        for (int o = 0; o < 16; ++o) acc[o] = fmaf(ws[(t * 16 + o) * 2], i2.x, fmaf(ws[(t * 16 + o) * 2 + 1], i2.y, acc[o]));
    }
#pragma unroll
    for (int o = 0; o < 16; ++o) acc[o] = fmaxf(acc[o], 0.f);
    store16_bf16(out + v * 16, acc);
}

// out = conv(a, w), a BF16 [V][16], w FP32 [27][1][16], out FP32 [V].
__global__ void conv_last_kernel(ConvGrid g, const __nv_bfloat16* __restrict__ a, const float* __restrict__ w,
                                 float* __restrict__ out) {
    __shared__ float ws[27 * 16];
    for (int i = threadIdx.x; i < 27 * 16; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    const long V = long(g.X) * g.Y * g.Z;
    const long v = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const Coord c = coord(v, g);
    float acc = 0.f;
    for (int t = 0; t < 27; ++t) {
        long nv;
        if (!neighbour(c, t, g, 1, &nv)) continue;
        float f[16];
        load8(a + nv * 16, f);
        load8(a + nv * 16 + 8, f + 8);
#pragma unroll
        for (int i = 0; i < 16; ++i) acc = fmaf(ws[t * 16 + i], f[i], acc);
    }
    out[v] = acc;
}

// g_a[v][c] = sum_t g_out[v - off_t] w[t][0][c]  (input gradient of conv_last).
__global__ void conv_last_backward_kernel(ConvGrid g, const float* __restrict__ gout, const float* __restrict__ w,
                                          float* __restrict__ ga) {
    __shared__ float ws[27 * 16];
    for (int i = threadIdx.x; i < 27 * 16; i += blockDim.x) ws[i] = w[i];
    __syncthreads();
    const long V = long(g.X) * g.Y * g.Z;
    const long v = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const Coord c = coord(v, g);
    float acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.f;
    for (int t = 0; t < 27; ++t) {
        long nv;
        if (!neighbour(c, t, g, -1, &nv)) continue;
        const float go = gout[nv];
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[i] = fmaf(ws[t * 16 + i], go, acc[i]);
    }
    float4* o = reinterpret_cast<float4*>(ga + v * 16);
#pragma unroll
    for (int i = 0; i < 4; ++i) o[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
}

// 2x2x2 average pooling of a BF16 [V][C] volume on grid g (the fine grid).
__global__ void pool_kernel(ConvGrid g, int C, const __nv_bfloat16* __restrict__ fine,
                            __nv_bfloat16* __restrict__ coarse) {
    const ConvGrid h{g.X / 2, g.Y / 2, g.Z / 2};
    const long Vc = long(h.X) * h.Y * h.Z;
    const int groups = C / 8;
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= Vc * groups) return;
    const long vc = i / groups;
    const int q = int(i % groups);
    const Coord c = coord(vc, h);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < 8; ++k) {
        const long vf = (long(2 * c.z + (k >> 2)) * g.Y + 2 * c.y + ((k >> 1) & 1)) * g.X + 2 * c.x + (k & 1);
        float f[8];
        load8(fine + vf * C + 8 * q, f);
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] += f[j];
    }
    __nv_bfloat162 hh[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) hh[j] = __floats2bfloat162_rn(0.125f * s[2 * j], 0.125f * s[2 * j + 1]);
    *reinterpret_cast<uint4*>(coarse + vc * C + 8 * q) = *reinterpret_cast<uint4*>(hh);
}

// h = bf16(g * (a > 0)), g FP32 [n], a BF16 [n].
__global__ void relu_mask_kernel(long n, const float* __restrict__ gr, const __nv_bfloat16* __restrict__ a,
                                 __nv_bfloat16* __restrict__ h) {
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    h[i] = __float2bfloat16_rn(bf(a[i]) > 0.f ? gr[i] : 0.f);
}

// Splits the gradient of a concatenated decoder input [up(coarse), skip]:
// g_skip[v][c] += g_cat[v][C1 + c]; g_coarse[vc][c] = sum over the 8 fine
// children of g_cat[child][c].
__global__ void split_cat_kernel(ConvGrid g, int C1, int C2, const float* __restrict__ gcat,
                                 float* __restrict__ gskip, float* __restrict__ gcoarse) {
    const ConvGrid h{g.X / 2, g.Y / 2, g.Z / 2};
    const long Vc = long(h.X) * h.Y * h.Z;
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= Vc) return;
    const Coord c = coord(i, h);
    const int C = C1 + C2;
    for (int ch = 0; ch < C1; ++ch) {
        float s = 0.f;
        for (int k = 0; k < 8; ++k) {
            const long vf = (long(2 * c.z + (k >> 2)) * g.Y + 2 * c.y + ((k >> 1) & 1)) * g.X + 2 * c.x + (k & 1);
            s += gcat[vf * C + ch];
        }
        gcoarse[i * C1 + ch] = s;
    }
    for (int k = 0; k < 8; ++k) {
        const long vf = (long(2 * c.z + (k >> 2)) * g.Y + 2 * c.y + ((k >> 1) & 1)) * g.X + 2 * c.x + (k & 1);
        for (int ch = 0; ch < C2; ++ch) gskip[vf * C2 + ch] += gcat[vf * C + C1 + ch];
    }
}

// g_fine[v][c] += g_coarse[parent(v)][c] / 8  (average pooling backward).
__global__ void pool_backward_kernel(ConvGrid g, int C, const float* __restrict__ gcoarse, float* __restrict__ gfine) {
    const long V = long(g.X) * g.Y * g.Z;
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= V * C) return;
    const long v = i / C;
    const int ch = int(i % C);
    const Coord c = coord(v, g);
    const long vc = (long(c.z >> 1) * (g.Y >> 1) + (c.y >> 1)) * (g.X >> 1) + (c.x >> 1);
    gfine[i] += 0.125f * gcoarse[vc * C + ch];
}

// Weight gradient dW[t][co][ci] += sum_v h[v][co] x[v + off_t][ci] on the CUDA
// cores.  h is BF16 [V][COUT] (or FP32 [V] for COUT = 1), x is either the
// concatenation of two BF16 sources (ConvSrc semantics) or FP32 [V][CIN].
// Each thread owns P = COUT*CIN/256 (co, ci) pairs of one co row; a block
// stages 128 voxels of h and of x's tap-shifted rows in shared memory.
template <int CIN, int COUT, bool XF, bool HF>
__global__ void __launch_bounds__(256) dw_kernel(ConvGrid g, const void* hp, ConvSrc s1, ConvSrc s2,
                                                 const float* xf, float* __restrict__ dw) {
    constexpr int kPairs = COUT * CIN;
    constexpr int P = kPairs >= 256 ? kPairs / 256 : 1;
    static_assert(kPairs < 256 || kPairs % 256 == 0, "pairs must tile the block");
    static_assert(kPairs < 256 || CIN % P == 0, "a thread's pairs must share one co");
    extern __shared__ float sm[];
    float* sx = sm;                  // [128][CIN]
    float* sh = sm + 128 * CIN;      // [128][COUT]
    const int tid = threadIdx.x;
    const long V = long(g.X) * g.Y * g.Z;
    const long tiles = V / 128;
    const int q0 = tid * P;
    const bool active = q0 < kPairs;
    const int co = active ? q0 / CIN : 0, ci0 = active ? q0 % CIN : 0;
    for (int t = 0; t < 27; ++t) {
        float acc[P];
#pragma unroll
        for (int k = 0; k < P; ++k) acc[k] = 0.f;
        for (long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
            __syncthreads();
            // stage h rows
            for (int i = tid; i < 128 * COUT; i += 256) {
                const long v = tile * 128 + i / COUT;
                const int c = i % COUT;
                sh[i] = HF ? static_cast<const float*>(hp)[v * COUT + c]
                           : bf(static_cast<const __nv_bfloat16*>(hp)[v * COUT + c]);
            }
            // stage x rows shifted by tap t
            for (int i = tid; i < 128 * CIN; i += 256) {
                const int r = i / CIN, c = i % CIN;
                const long v = tile * 128 + r;
                const Coord cc = coord(v, g);
                long nv;
                float val = 0.f;
                if (neighbour(cc, t, g, 1, &nv)) {
                    if (XF) {
                        val = xf[nv * CIN + c];
                    } else {
                        const Coord nc = coord(nv, g);
                        if (c < s1.C) {
                            const long idx = s1.up ? (long(nc.z >> 1) * (g.Y >> 1) + (nc.y >> 1)) * (g.X >> 1) + (nc.x >> 1)
                                                   : nv;
                            val = bf(s1.p[idx * s1.C + c]);
                        } else {
                            val = bf(s2.p[nv * s2.C + (c - s1.C)]);
                        }
                    }
                }
                sx[i] = val;
            }
            __syncthreads();
            if (active) {
                for (int r = 0; r < 128; ++r) {
                    const float hv = sh[r * COUT + co];
#pragma unroll
                    for (int k = 0; k < P; ++k) acc[k] = fmaf(hv, sx[r * CIN + ci0 + k], acc[k]);
                }
            }
        }
        if (active) {
#pragma unroll
            for (int k = 0; k < P; ++k)
                if (q0 + k < kPairs) atomicAdd(&dw[(size_t(t) * COUT + co) * CIN + ci0 + k], acc[k]);
        }
    }
}

// Adam (Kingma & Ba 2015) on one parameter array.
__global__ void adam_kernel(long n, float* __restrict__ w, const float* __restrict__ gr, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps) {
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 packs of a tensor-core layer: forward [t][co][ci] and the transposed,
// flipped kernel of the input gradient [26 - t][ci][co].
__global__ void pack_kernel(int cin, int cout, const float* __restrict__ w, __nv_bfloat16* __restrict__ wf,
                            __nv_bfloat16* __restrict__ wt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = 27 * cout * cin;
    if (i >= n) return;
    const int t = i / (cout * cin), co = (i / cin) % cout, ci = i % cin;
    const __nv_bfloat16 h = __float2bfloat16_rn(w[i]);
    wf[i] = h;
    wt[(size_t(26 - t) * cin + ci) * cout + co] = h;
}

// Loss of one sample: L = sum m (out - t)^2 / sum m t^2 (the relative error
// of the predicted potential increment over the mesh cells).
__global__ void loss_sums_kernel(long n, const float* __restrict__ out, const float* __restrict__ tgt,
                                 const float* __restrict__ mask, double* sums) {
    __shared__ double s0[256], s1[256];
    double a = 0.0, b = 0.0;
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const double mm = mask[i], d = double(out[i]) - tgt[i];
        a += mm * d * d;
        b += mm * double(tgt[i]) * tgt[i];
    }
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = b;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(sums, s0[0]);
        atomicAdd(sums + 1, s1[0]);
    }
}

__global__ void loss_grad_kernel(long n, const float* __restrict__ out, const float* __restrict__ tgt,
                                 const float* __restrict__ mask, const double* sums, float* __restrict__ gout) {
    const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double den = sums[1] > 0 ? sums[1] : 1.0;
    gout[i] = float(2.0 * mask[i] * (double(out[i]) - tgt[i]) / den);
}

template <class T>
cudaError_t zero(T* p, size_t n, cudaStream_t s) {
    return cudaMemsetAsync(p, 0, n * sizeof(T), s);
}

unsigned nblk(long n, int bs = 256) { return unsigned((n + bs - 1) / bs); }

template <int CIN, int COUT, bool XF, bool HF>
void launch_dw(const ConvGrid& g, const void* h, const ConvSrc& s1, const ConvSrc& s2, const float* xf, float* dw,
               cudaStream_t s) {
    const long tiles = long(g.X) * g.Y * g.Z / 128;
    const int smem = 128 * (CIN + COUT) * int(sizeof(float));
    auto k = dw_kernel<CIN, COUT, XF, HF>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k<<<unsigned(std::min<long>(tiles, 1216)), 256, smem, s>>>(g, h, s1, s2, xf, dw);
}

}  // namespace

// ------------------------------------------------------------------ UNet --
UNet::~UNet() { release(); }

void UNet::release() {
    for (void* p : allocs_) cudaFree(p);
    allocs_.clear();
}

template <class T>
T* UNet::alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    allocs_.push_back(p);
    return static_cast<T*>(p);
}

bool UNet::grid_supported(int X, int Y, int Z) {
    if (X % 4 || Y % 4 || Z % 4 || X <= 0 || Y <= 0 || Z <= 0) return false;
    const long V = long(X) * Y * Z;
    return V % 128 == 0 && (V / 8) % 128 == 0 && (V / 64) % 128 == 0;
}

size_t UNet::param_count() {
    size_t n = 0;
    for (int l = 0; l < kUNetNumLayers; ++l) n += size_t(27) * kUNetLayers[l].cin * kUNetLayers[l].cout;
    return n;
}

int UNet::init(int X, int Y, int Z, uint64_t seed, std::string* msg) {
    if (!grid_supported(X, Y, Z)) {
        *msg = "learned warm start: grid must be a multiple of 4 per direction with (X*Y*Z)/64 a multiple of 128";
        return 1;
    }
    g1_ = {X, Y, Z};
    g2_ = {X / 2, Y / 2, Z / 2};
    g3_ = {X / 4, Y / 4, Z / 4};
    const long V1 = long(X) * Y * Z, V2 = V1 / 8, V3 = V1 / 64;
    V1_ = V1;
    nparam_ = param_count();
    // parameters: master, gradient, Adam moments (one flat array each)
    w_ = alloc<float>(nparam_);
    gw_ = alloc<float>(nparam_);
    m_ = alloc<float>(nparam_);
    v_ = alloc<float>(nparam_);
    size_t off = 0;
    size_t pack = 0;
    for (int l = 0; l < kUNetNumLayers; ++l) {
        off_[l] = off;
        off += size_t(27) * kUNetLayers[l].cin * kUNetLayers[l].cout;
    }
    for (int l = 1; l <= 9; ++l) pack += size_t(27) * kUNetLayers[l].cin * kUNetLayers[l].cout;
    wf_all_ = alloc<__nv_bfloat16>(pack);
    wt_all_ = alloc<__nv_bfloat16>(pack);
    size_t po = 0;
    for (int l = 1; l <= 9; ++l) {
        wf_[l] = wf_all_ + po;
        wt_[l] = wt_all_ + po;
        po += size_t(27) * kUNetLayers[l].cin * kUNetLayers[l].cout;
    }
    // activations
    in_ = alloc<float>(2 * V1);
    a_[1] = alloc<__nv_bfloat16>(16 * V1);
    a_[2] = alloc<__nv_bfloat16>(16 * V1);
    p1_ = alloc<__nv_bfloat16>(16 * V2);
    a_[3] = alloc<__nv_bfloat16>(32 * V2);
    a_[4] = alloc<__nv_bfloat16>(32 * V2);
    p2_ = alloc<__nv_bfloat16>(32 * V3);
    a_[5] = alloc<__nv_bfloat16>(64 * V3);
    a_[6] = alloc<__nv_bfloat16>(64 * V3);
    a_[7] = alloc<__nv_bfloat16>(32 * V2);
    a_[8] = alloc<__nv_bfloat16>(32 * V2);
    a_[9] = alloc<__nv_bfloat16>(16 * V1);
    a_[10] = alloc<__nv_bfloat16>(16 * V1);
    out_ = alloc<float>(V1);
    // backward scratch: FP32 gradients (largest: 48 channels at V1), BF16 masked copy
    gA_ = alloc<float>(48 * V1);
    gB_ = alloc<float>(16 * V1);
    gskip1_ = alloc<float>(16 * V1);
    gskip2_ = alloc<float>(32 * V2);
    gC_ = alloc<float>(64 * V2);
    hb_ = alloc<__nv_bfloat16>(32 * V1);
    gout_ = alloc<float>(V1);
    sums_ = alloc<double>(2);
    err_ = alloc<int>(1);
    if (!w_ || !gw_ || !m_ || !v_ || !wf_all_ || !wt_all_ || !in_ || !a_[1] || !a_[2] || !p1_ || !a_[3] || !a_[4] ||
        !p2_ || !a_[5] || !a_[6] || !a_[7] || !a_[8] || !a_[9] || !a_[10] || !out_ || !gA_ || !gB_ || !gskip1_ ||
        !gskip2_ || !gC_ || !hb_ || !gout_ || !sums_ || !err_) {
        *msg = "learned warm start: device allocation failed";
        return 2;
    }
    if (cudaMemset(err_, 0, sizeof(int)) != cudaSuccess || cudaMemset(sums_, 0, 2 * sizeof(double)) != cudaSuccess) {
        *msg = "learned warm start: device memset failed";
        return 3;
    }
    // He-normal initialisation from a fixed splitmix64 / Box-Muller stream
    std::vector<float> h(nparam_);
    uint64_t st = seed ^ 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (int l = 0; l < kUNetNumLayers; ++l) {
        const int cin = kUNetLayers[l].cin, cout = kUNetLayers[l].cout;
        const double sd = std::sqrt((l == kUNetNumLayers - 1 ? 1.0 : 2.0) / (27.0 * cin));
        for (size_t i = 0; i < size_t(27) * cin * cout; ++i) {
            const double u1 = (double(next() >> 11) + 1.0) * (1.0 / 9007199254740992.0);
            const double u2 = double(next() >> 11) * (1.0 / 9007199254740992.0);
            h[off_[l] + i] = float(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    if (set_weights(h.data(), 0) != cudaSuccess) {
        *msg = "learned warm start: weight upload failed";
        return 3;
    }
    return 0;
}

cudaError_t UNet::set_weights(const float* host, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(w_, host, nparam_ * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    zero(m_, nparam_, s);
    zero(v_, nparam_, s);
    adam_t_ = 0;
    pack(s);
    return cudaStreamSynchronize(s);
}

cudaError_t UNet::get_weights(float* host, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(host, w_, nparam_ * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

cudaError_t UNet::get_gradients(float* host, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(host, gw_, nparam_ * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

void UNet::pack(cudaStream_t s) {
    for (int l = 1; l <= 9; ++l) {
        const int n = 27 * kUNetLayers[l].cin * kUNetLayers[l].cout;
        pack_kernel<<<nblk(n), 256, 0, s>>>(kUNetLayers[l].cin, kUNetLayers[l].cout, w_ + off_[l], wf_[l], wt_[l]);
    }
}

cudaError_t UNet::tc(int l, int epi, const ConvGrid& g, ConvSrc s1, ConvSrc s2, void* out, cudaStream_t s) {
    return launch_conv_tc(kUNetLayers[l].cin, kUNetLayers[l].cout, epi, g, s1, s2, wf_[l], out, err_, s);
}

cudaError_t UNet::forward(cudaStream_t s) {
    const ConvSrc none{nullptr, 0, 0};
    cudaError_t e;
    conv_first_kernel<<<nblk(V1_), 256, 0, s>>>(g1_, in_, w_ + off_[0], a_[1]);
    launches_ += 1;
    if ((e = tc(1, kEpiReluBf16, g1_, {a_[1], 16, 0}, none, a_[2], s))) return e;
    pool_kernel<<<nblk(V1_ / 8 * 2), 256, 0, s>>>(g1_, 16, a_[2], p1_);
    if ((e = tc(2, kEpiReluBf16, g2_, {p1_, 16, 0}, none, a_[3], s))) return e;
    if ((e = tc(3, kEpiReluBf16, g2_, {a_[3], 32, 0}, none, a_[4], s))) return e;
    pool_kernel<<<nblk(V1_ / 64 * 4), 256, 0, s>>>(g2_, 32, a_[4], p2_);
    if ((e = tc(4, kEpiReluBf16, g3_, {p2_, 32, 0}, none, a_[5], s))) return e;
    if ((e = tc(5, kEpiReluBf16, g3_, {a_[5], 64, 0}, none, a_[6], s))) return e;
    if ((e = tc(6, kEpiReluBf16, g2_, {a_[6], 64, 1}, {a_[4], 32, 0}, a_[7], s))) return e;
    if ((e = tc(7, kEpiReluBf16, g2_, {a_[7], 32, 0}, none, a_[8], s))) return e;
    if ((e = tc(8, kEpiReluBf16, g1_, {a_[8], 32, 1}, {a_[2], 16, 0}, a_[9], s))) return e;
    if ((e = tc(9, kEpiReluBf16, g1_, {a_[9], 16, 0}, none, a_[10], s))) return e;
    conv_last_kernel<<<nblk(V1_), 256, 0, s>>>(g1_, a_[10], w_ + off_[10], out_);
    launches_ += 13;
    return cudaGetLastError();
}

// Input gradient of tensor-core layer l (FP32 out) from the masked BF16
// output gradient hb_ (cout channels).
cudaError_t UNet::tc_dx(int l, const ConvGrid& g, float* gin, cudaStream_t s) {
    const ConvSrc none{nullptr, 0, 0};
    const int cin = kUNetLayers[l].cin, cout = kUNetLayers[l].cout;
    launches_ += 1;
    return launch_conv_tc(cout, cin, kEpiF32, g, {hb_, cout, 0}, none, wt_[l], gin, err_, s);
}

void UNet::mask(const float* gr, const __nv_bfloat16* a, long n, cudaStream_t s) {
    relu_mask_kernel<<<nblk(n), 256, 0, s>>>(n, gr, a, hb_);
    launches_ += 1;
}

cudaError_t UNet::backward(cudaStream_t s) {
    const ConvSrc none{nullptr, 0, 0};
    const long V2 = V1_ / 8, V3 = V1_ / 64;
    float* g = gw_;
    cudaError_t e;
    zero(gw_, nparam_, s);
    // out = co(a10)
    launch_dw<16, 1, false, true>(g1_, gout_, {a_[10], 16, 0}, none, nullptr, g + off_[10], s);
    conv_last_backward_kernel<<<nblk(V1_), 256, 0, s>>>(g1_, gout_, w_ + off_[10], gB_);
    // a10 = relu(d1b(a9))
    mask(gB_, a_[10], 16 * V1_, s);
    launch_dw<16, 16, false, false>(g1_, hb_, {a_[9], 16, 0}, none, nullptr, g + off_[9], s);
    if ((e = tc_dx(9, g1_, gB_, s))) return e;  // g_a9
    // a9 = relu(d1a([up(a8), a2]))
    mask(gB_, a_[9], 16 * V1_, s);
    launch_dw<48, 16, false, false>(g1_, hb_, {a_[8], 32, 1}, {a_[2], 16, 0}, nullptr, g + off_[8], s);
    if ((e = tc_dx(8, g1_, gA_, s))) return e;  // g_cat [V1][48]
    zero(gskip1_, 16 * size_t(V1_), s);
    split_cat_kernel<<<nblk(V2), 256, 0, s>>>(g1_, 32, 16, gA_, gskip1_, gC_);  // g_a8 -> gC_ [V2][32]
    // a8 = relu(d2b(a7))
    mask(gC_, a_[8], 32 * V2, s);
    launch_dw<32, 32, false, false>(g2_, hb_, {a_[7], 32, 0}, none, nullptr, g + off_[7], s);
    if ((e = tc_dx(7, g2_, gB_, s))) return e;  // g_a7 [V2][32]
    // a7 = relu(d2a([up(a6), a4]))
    mask(gB_, a_[7], 32 * V2, s);
    launch_dw<96, 32, false, false>(g2_, hb_, {a_[6], 64, 1}, {a_[4], 32, 0}, nullptr, g + off_[6], s);
    if ((e = tc_dx(6, g2_, gA_, s))) return e;  // g_cat [V2][96]
    zero(gskip2_, 32 * size_t(V2), s);
    split_cat_kernel<<<nblk(V3), 256, 0, s>>>(g2_, 64, 32, gA_, gskip2_, gC_);  // g_a6 -> gC_ [V3][64]
    // a6 = relu(c3b(a5))
    mask(gC_, a_[6], 64 * V3, s);
    launch_dw<64, 64, false, false>(g3_, hb_, {a_[5], 64, 0}, none, nullptr, g + off_[5], s);
    if ((e = tc_dx(5, g3_, gB_, s))) return e;  // g_a5 [V3][64]
    // a5 = relu(c3a(p2))
    mask(gB_, a_[5], 64 * V3, s);
    launch_dw<32, 64, false, false>(g3_, hb_, {p2_, 32, 0}, none, nullptr, g + off_[4], s);
    if ((e = tc_dx(4, g3_, gC_, s))) return e;  // g_p2 [V3][32]
    pool_backward_kernel<<<nblk(32 * V2), 256, 0, s>>>(g2_, 32, gC_, gskip2_);  // g_a4 total
    // a4 = relu(c2b(a3))
    mask(gskip2_, a_[4], 32 * V2, s);
    launch_dw<32, 32, false, false>(g2_, hb_, {a_[3], 32, 0}, none, nullptr, g + off_[3], s);
    if ((e = tc_dx(3, g2_, gB_, s))) return e;  // g_a3 [V2][32]
    // a3 = relu(c2a(p1))
    mask(gB_, a_[3], 32 * V2, s);
    launch_dw<16, 32, false, false>(g2_, hb_, {p1_, 16, 0}, none, nullptr, g + off_[2], s);
    if ((e = tc_dx(2, g2_, gC_, s))) return e;  // g_p1 [V2][16]
    pool_backward_kernel<<<nblk(16 * V1_), 256, 0, s>>>(g1_, 16, gC_, gskip1_);  // g_a2 total
    // a2 = relu(c1b(a1))
    mask(gskip1_, a_[2], 16 * V1_, s);
    launch_dw<16, 16, false, false>(g1_, hb_, {a_[1], 16, 0}, none, nullptr, g + off_[1], s);
    if ((e = tc_dx(1, g1_, gB_, s))) return e;  // g_a1
    // a1 = relu(c1a(in))
    mask(gB_, a_[1], 16 * V1_, s);
    launch_dw<2, 16, true, false>(g1_, hb_, none, none, in_, g + off_[0], s);
    launches_ += 30;
    return cudaGetLastError();
}

cudaError_t UNet::loss_and_grad(const float* target, const float* maskv, cudaStream_t s) {
    zero(sums_, 2, s);
    loss_sums_kernel<<<std::min<unsigned>(nblk(V1_), 1216), 256, 0, s>>>(V1_, out_, target, maskv, sums_);
    loss_grad_kernel<<<nblk(V1_), 256, 0, s>>>(V1_, out_, target, maskv, sums_, gout_);
    launches_ += 2;
    return cudaGetLastError();
}

cudaError_t UNet::adam(float lr, cudaStream_t s) {
    ++adam_t_;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, float(adam_t_)), c2 = 1.f - std::pow(b2, float(adam_t_));
    adam_kernel<<<nblk(long(nparam_)), 256, 0, s>>>(long(nparam_), w_, gw_, m_, v_, lr, b1, b2, c1, c2, 1e-8f);
    pack(s);
    launches_ += 1 + 9;
    return cudaGetLastError();
}

cudaError_t UNet::read_loss(double* loss, cudaStream_t s) {
    double h[2];
    cudaError_t e = cudaMemcpyAsync(h, sums_, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    *loss = h[1] > 0 ? h[0] / h[1] : 0.0;
    return cudaSuccess;
}

cudaError_t UNet::check_error(bool* timed_out, cudaStream_t s) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, err_, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    *timed_out = h != 0;
    return e;
}

}  // namespace pgd
