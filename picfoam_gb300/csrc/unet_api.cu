// unet_api.cu -- C ABI of the learned warm start (include/picgpu_learned.h).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "picgpu_learned.h"
#include "unet.h"

namespace {

struct DeviceBuffers {
    std::vector<void*> ptrs;
    ~DeviceBuffers() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

}  // namespace

extern "C" picgpu_status picgpu_test_conv3d(int X, int Y, int Z, int cin1, int cin2, int up1, int cout, int relu,
                                            const uint16_t* in1, const uint16_t* in2, const uint16_t* w,
                                            float* out) {
    if (X <= 0 || Y <= 0 || Z <= 0 || cin1 <= 0 || cin2 < 0 || !in1 || (cin2 > 0 && !in2) || !w || !out)
        return PICGPU_INVALID_ARG;
    const long V = long(X) * Y * Z;
    if (V % 128 != 0 || cin1 % 8 != 0 || cin2 % 8 != 0 || (up1 && (X % 2 || Y % 2 || Z % 2)))
        return PICGPU_INVALID_ARG;
    const int cin = cin1 + cin2;
    if (!pgd::conv_tc_supported(cin, cout)) return PICGPU_NOT_SUPPORTED;
    const long V1 = up1 ? V / 8 : V;
    DeviceBuffers B;
    auto* d1 = B.alloc<__nv_bfloat16>(size_t(V1) * cin1);
    auto* d2 = cin2 > 0 ? B.alloc<__nv_bfloat16>(size_t(V) * cin2) : nullptr;
    auto* dw = B.alloc<__nv_bfloat16>(size_t(27) * cout * cin);
    void* dout = relu ? static_cast<void*>(B.alloc<__nv_bfloat16>(size_t(V) * cout))
                      : static_cast<void*>(B.alloc<float>(size_t(V) * cout));
    int* derr = B.alloc<int>(1);
    if (!d1 || (cin2 > 0 && !d2) || !dw || !dout || !derr) return PICGPU_OOM;
    if (cudaMemcpy(d1, in1, size_t(V1) * cin1 * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
        (cin2 > 0 && cudaMemcpy(d2, in2, size_t(V) * cin2 * 2, cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemcpy(dw, w, size_t(27) * cout * cin * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(derr, 0, sizeof(int)) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    pgd::ConvGrid g{X, Y, Z};
    pgd::ConvSrc s1{d1, cin1, up1}, s2{d2, cin2, 0};
    if (pgd::launch_conv_tc(cin, cout, relu ? pgd::kEpiReluBf16 : pgd::kEpiF32, g, s1, s2, dw, dout, derr, 0) !=
        cudaSuccess)
        return PICGPU_CUDA_ERROR;
    int herr = 0;
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    if (herr) return PICGPU_CUDA_ERROR;
    if (relu) {
        std::vector<uint16_t> h(size_t(V) * cout);
        if (cudaMemcpy(h.data(), dout, h.size() * 2, cudaMemcpyDeviceToHost) != cudaSuccess) return PICGPU_CUDA_ERROR;
        for (size_t i = 0; i < h.size(); ++i) {
            const uint32_t bits = uint32_t(h[i]) << 16;
            float f;
            std::memcpy(&f, &bits, 4);
            out[i] = f;
        }
    } else if (cudaMemcpy(out, dout, size_t(V) * cout * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        return PICGPU_CUDA_ERROR;
    }
    return PICGPU_OK;
}
