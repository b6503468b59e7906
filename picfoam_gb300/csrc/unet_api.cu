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

// --------------------------------------------------------- the network --
#include <memory>

#include "unet_net.h"

struct picgpu_unet {
    pgd::UNet net;
    cudaStream_t stream = nullptr;
    float* target = nullptr;
    float* mask = nullptr;
};

namespace {

picgpu_status upload_sample(picgpu_unet* u, const float* in, const float* target, const float* mask) {
    const long V = u->net.voxels();
    cudaStream_t s = u->stream;
    if (cudaMemcpyAsync(u->net.input(), in, size_t(V) * 2 * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    if (target && cudaMemcpyAsync(u->target, target, size_t(V) * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    if (mask && cudaMemcpyAsync(u->mask, mask, size_t(V) * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    return PICGPU_OK;
}

picgpu_status finish(picgpu_unet* u) {
    bool timed_out = false;
    if (cudaGetLastError() != cudaSuccess || u->net.check_error(&timed_out, u->stream) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    return timed_out ? PICGPU_CUDA_ERROR : PICGPU_OK;
}

}  // namespace

extern "C" {

size_t picgpu_unet_param_count(void) { return pgd::UNet::param_count(); }

picgpu_status picgpu_unet_create(int X, int Y, int Z, uint64_t seed, picgpu_unet** out) {
    if (!out) return PICGPU_INVALID_ARG;
    *out = nullptr;
    if (!pgd::UNet::grid_supported(X, Y, Z)) return PICGPU_INVALID_ARG;
    auto u = std::make_unique<picgpu_unet>();
    std::string msg;
    if (cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking) != cudaSuccess) return PICGPU_CUDA_ERROR;
    const int e = u->net.init(X, Y, Z, seed, &msg);
    if (e) {
        cudaStreamDestroy(u->stream);
        return e == 2 ? PICGPU_OOM : PICGPU_CUDA_ERROR;
    }
    const long V = long(X) * Y * Z;
    if (cudaMalloc(&u->target, size_t(V) * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&u->mask, size_t(V) * sizeof(float)) != cudaSuccess) {
        cudaFree(u->target);
        cudaStreamDestroy(u->stream);
        return PICGPU_OOM;
    }
    *out = u.release();
    return PICGPU_OK;
}

void picgpu_unet_destroy(picgpu_unet* u) {
    if (!u) return;
    cudaStreamSynchronize(u->stream);
    cudaFree(u->target);
    cudaFree(u->mask);
    cudaStreamDestroy(u->stream);
    delete u;
}

picgpu_status picgpu_unet_set_weights(picgpu_unet* u, const float* w) {
    if (!u || !w) return PICGPU_INVALID_ARG;
    return u->net.set_weights(w, u->stream) == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

picgpu_status picgpu_unet_get_weights(picgpu_unet* u, float* w) {
    if (!u || !w) return PICGPU_INVALID_ARG;
    return u->net.get_weights(w, u->stream) == cudaSuccess ? PICGPU_OK : PICGPU_CUDA_ERROR;
}

picgpu_status picgpu_unet_forward(picgpu_unet* u, const float* in, float* out) {
    if (!u || !in || !out) return PICGPU_INVALID_ARG;
    picgpu_status st = upload_sample(u, in, nullptr, nullptr);
    if (st) return st;
    if (u->net.forward(u->stream) != cudaSuccess) return PICGPU_CUDA_ERROR;
    if (cudaMemcpyAsync(out, u->net.output(), size_t(u->net.voxels()) * sizeof(float), cudaMemcpyDeviceToHost,
                        u->stream) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    return finish(u);
}

picgpu_status picgpu_unet_gradients(picgpu_unet* u, const float* in, const float* target, const float* mask,
                                    float* grad, double* loss) {
    if (!u || !in || !target || !mask || !grad) return PICGPU_INVALID_ARG;
    picgpu_status st = upload_sample(u, in, target, mask);
    if (st) return st;
    if (u->net.forward(u->stream) != cudaSuccess || u->net.loss_and_grad(u->target, u->mask, u->stream) != cudaSuccess ||
        u->net.backward(u->stream) != cudaSuccess)
        return PICGPU_CUDA_ERROR;
    if ((st = finish(u))) return st;
    if (u->net.get_gradients(grad, u->stream) != cudaSuccess) return PICGPU_CUDA_ERROR;
    if (loss && u->net.read_loss(loss, u->stream) != cudaSuccess) return PICGPU_CUDA_ERROR;
    return PICGPU_OK;
}

picgpu_status picgpu_unet_train(picgpu_unet* u, const float* in, const float* target, const float* mask, int iters,
                                double lr, double* loss) {
    if (!u || !in || !target || !mask || iters < 0 || !(lr > 0)) return PICGPU_INVALID_ARG;
    picgpu_status st = upload_sample(u, in, target, mask);
    if (st) return st;
    for (int k = 0; k < iters; ++k) {
        if (u->net.forward(u->stream) != cudaSuccess ||
            u->net.loss_and_grad(u->target, u->mask, u->stream) != cudaSuccess ||
            u->net.backward(u->stream) != cudaSuccess || u->net.adam(float(lr), u->stream) != cudaSuccess)
            return PICGPU_CUDA_ERROR;
    }
    if ((st = finish(u))) return st;
    if (loss && u->net.read_loss(loss, u->stream) != cudaSuccess) return PICGPU_CUDA_ERROR;
    return PICGPU_OK;
}

}  // extern "C"
