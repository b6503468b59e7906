// unet_conv.cu -- 3x3x3 "same" convolution on the 5th-generation tensor cores.
//
// Implicit GEMM: a CTA owns 128 consecutive voxels of a channels-last BF16
// volume (the MMA's M = 128) and all C_out output channels (N); K runs over
// the 27 taps x C_in channels.  Per tap the 128 input rows (zero outside the
// volume) and the tap's C_out x C_in weight slice are staged in shared
// memory as K-major core matrices (tc.cuh) by all threads, then one thread
// issues C_in / 16 tcgen05.mma (K = 16 each) into an FP32 accumulator in TMEM
// and commits them to the stage's mbarrier.  Two stages: the loads of tap
// t + 1 overlap the MMAs of tap t.  The epilogue reads the accumulator with
// tcgen05.ld (lane = voxel row) and stores either ReLU -> BF16 or raw FP32.
//
// The input may be the concatenation of two channels-last sources, the first
// optionally at half resolution (nearest-neighbour upsampling), which is how
// the decoder reads [up(coarse), skip] without materialising it.
//
// Every mbarrier wait is bounded; on a timeout the kernel raises *err, skips
// the rest of its work, frees its TMEM and returns.
#include <cuda_bf16.h>

#include "tc.cuh"
#include "unet.h"

namespace pgd {
namespace {

constexpr int kRows = 128;                    // voxels per CTA
constexpr uint32_t kAKStride = (kRows / 8) * 128;  // bytes between K-adjacent core matrices of A
constexpr int kGuard = 32768;                 // slack behind the stages (descriptor safety margin)

template <int CIN, int COUT>
struct ConvShape {
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT >= 16 && COUT <= 256, "unsupported channel counts");
    static constexpr int kABytes = kRows * CIN * 2;
    static constexpr int kBBytes = COUT * CIN * 2;
    static constexpr int kStage = kABytes + kBBytes;
    static constexpr int kSmem = 2 * kStage + kGuard;
    static constexpr uint32_t kBKStride = (COUT / 8) * 128;
    static constexpr uint32_t kCols = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : (COUT <= 128 ? 128 : 256));
};

// Stage one source's channels of the row this thread owns.
__device__ __forceinline__ void stage_rows(const ConvSrc& s, int j0, bool inside, const ConvGrid& g, int xn, int yn,
                                           int zn, uint8_t* arow) {
    const int nv = s.C / 8;
    if (inside) {
        long idx;
        if (s.up) idx = (long(zn >> 1) * (g.Y >> 1) + (yn >> 1)) * (g.X >> 1) + (xn >> 1);
        else idx = (long(zn) * g.Y + yn) * g.X + xn;
        const uint4* src = reinterpret_cast<const uint4*>(s.p + idx * s.C);
        for (int j = 0; j < nv; ++j) *reinterpret_cast<uint4*>(arow + (j0 + j) * kAKStride) = __ldg(src + j);
    } else {
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        for (int j = 0; j < nv; ++j) *reinterpret_cast<uint4*>(arow + (j0 + j) * kAKStride) = z;
    }
}

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(128) conv_tc_kernel(ConvGrid g, ConvSrc s1, ConvSrc s2,
                                                      const __nv_bfloat16* __restrict__ w, void* out, int* err) {
    using S = ConvShape<CIN, COUT>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const long v = long(blockIdx.x) * kRows + tid;
    const long XY = long(g.X) * g.Y;
    const int x = int(v % g.X), y = int((v / g.X) % g.Y), z = int(v / XY);

    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        abort_flag = 0;
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, S::kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kRows, COUT);

    for (int t = 0; t < 27; ++t) {
        const int s = t & 1;
        uint8_t* A = smem + s * S::kStage;
        uint8_t* B = A + S::kABytes;
        // the MMAs of tap t - 2 read this stage: wait for them
        if (t >= 2 && !abort_flag && !tc::mbar_wait(&bar[s], uint32_t((t - 2) >> 1) & 1u)) abort_flag = 1;
        const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
        const int xn = x + dx, yn = y + dy, zn = z + dz;
        const bool inside = xn >= 0 && xn < g.X && yn >= 0 && yn < g.Y && zn >= 0 && zn < g.Z;
        uint8_t* arow = A + (tid >> 3) * 128 + (tid & 7) * 16;
        stage_rows(s1, 0, inside, g, xn, yn, zn, arow);
        if (s2.C > 0) stage_rows(s2, s1.C / 8, inside, g, xn, yn, zn, arow);
        const uint4* wt = reinterpret_cast<const uint4*>(w + size_t(t) * COUT * CIN);
        for (int q = tid; q < COUT * CIN / 8; q += 128) {
            const int co = q / (CIN / 8), j = q % (CIN / 8);
            *reinterpret_cast<uint4*>(B + j * S::kBKStride + (co >> 3) * 128 + (co & 7) * 16) = __ldg(wt + q);
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0 && !abort_flag) {
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_addr(A), b0 = tc::smem_addr(B);
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
                const uint64_t ad = tc::smem_desc(a0 + 2u * kc * kAKStride, kAKStride, 128);
                const uint64_t bd = tc::smem_desc(b0 + 2u * kc * S::kBKStride, S::kBKStride, 128);
                tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || kc > 0) ? 1u : 0u);
            }
            tc::commit(&bar[s]);
        }
    }
    // the commit of tap 26 (stage 0, its 14th use) covers every MMA before it
    if (!abort_flag && !tc::mbar_wait(&bar[0], 1u)) abort_flag = 1;
    __syncthreads();
    tc::fence_after_sync();
    if (!abort_flag) {
        const uint32_t lane_base = tmem + (uint32_t(warp * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tc::tmem_ld16(lane_base + uint32_t(c0), acc);
            if (EPI == kEpiReluBf16) {
                __nv_bfloat162 h[8];
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    h[i] = __floats2bfloat162_rn(fmaxf(acc[2 * i], 0.f), fmaxf(acc[2 * i + 1], 0.f));
                uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(out) + v * COUT + c0);
                o[0] = *reinterpret_cast<uint4*>(&h[0]);
                o[1] = *reinterpret_cast<uint4*>(&h[4]);
            } else {
                float4* o = reinterpret_cast<float4*>(static_cast<float*>(out) + v * COUT + c0);
#pragma unroll
                for (int i = 0; i < 4; ++i) o[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
            }
        }
    }
    if (abort_flag && tid == 0) atomicExch(err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, S::kCols);
}

template <int CIN, int COUT, int EPI>
cudaError_t launch(const ConvGrid& g, const ConvSrc& s1, const ConvSrc& s2, const __nv_bfloat16* w, void* out,
                   int* err, cudaStream_t st) {
    using S = ConvShape<CIN, COUT>;
    auto k = conv_tc_kernel<CIN, COUT, EPI>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem);
    if (e != cudaSuccess) return e;
    const long V = long(g.X) * g.Y * g.Z;
    k<<<unsigned(V / kRows), 128, S::kSmem, st>>>(g, s1, s2, w, out, err);
    return cudaGetLastError();
}

template <int EPI>
cudaError_t dispatch(int cin, int cout, const ConvGrid& g, const ConvSrc& s1, const ConvSrc& s2,
                     const __nv_bfloat16* w, void* out, int* err, cudaStream_t st) {
#define PGD_CONV(CI, CO) \
    if (cin == CI && cout == CO) return launch<CI, CO, EPI>(g, s1, s2, w, out, err, st);
    PGD_CONV(16, 16) PGD_CONV(16, 32) PGD_CONV(32, 16) PGD_CONV(32, 32) PGD_CONV(32, 64) PGD_CONV(64, 32)
    PGD_CONV(64, 64) PGD_CONV(96, 32) PGD_CONV(32, 96) PGD_CONV(48, 16) PGD_CONV(16, 48)
#undef PGD_CONV
    return cudaErrorInvalidValue;
}

}  // namespace

bool conv_tc_supported(int cin, int cout) {
    const int ok[][2] = {{16, 16}, {16, 32}, {32, 16}, {32, 32}, {32, 64}, {64, 32},
                         {64, 64}, {96, 32}, {32, 96}, {48, 16}, {16, 48}};
    for (auto& p : ok)
        if (p[0] == cin && p[1] == cout) return true;
    return false;
}

cudaError_t launch_conv_tc(int cin, int cout, int epi, const ConvGrid& g, const ConvSrc& s1, const ConvSrc& s2,
                           const __nv_bfloat16* w, void* out, int* err, cudaStream_t st) {
    const long V = long(g.X) * g.Y * g.Z;
    if (V <= 0 || V % kRows != 0 || s1.C + s2.C != cin || s1.C % 8 != 0 || s2.C % 8 != 0 ||
        (s1.up && (g.X % 2 || g.Y % 2 || g.Z % 2)) || s2.up)
        return cudaErrorInvalidValue;
    if (epi == kEpiReluBf16) return dispatch<kEpiReluBf16>(cin, cout, g, s1, s2, w, out, err, st);
    return dispatch<kEpiF32>(cin, cout, g, s1, s2, w, out, err, st);
}

}  // namespace pgd
