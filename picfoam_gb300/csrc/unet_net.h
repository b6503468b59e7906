// unet_net.h -- host-side driver of the warm-start U-Net (unet.cu).
#pragma once

#include "unet.h"

namespace pgd {

struct UNetLayerDef {
    int cin, cout;
};
constexpr int kUNetNumLayers = 11;
// c1a c1b c2a c2b c3a c3b d2a d2b d1a d1b co; weights FP32 [27][cout][cin]
// per layer, stored back to back in this order.
extern const UNetLayerDef kUNetLayers[kUNetNumLayers];

class UNet {
   public:
    UNet() = default;
    UNet(const UNet&) = delete;
    UNet& operator=(const UNet&) = delete;
    ~UNet();

    // Grids whose three levels tile into 128-voxel MMA blocks.
    static bool grid_supported(int X, int Y, int Z);
    static size_t param_count();

    // Allocates everything and draws He-normal weights; 0 on success.
    int init(int X, int Y, int Z, uint64_t seed, std::string* msg);

    long voxels() const { return V1_; }
    float* input() { return in_; }    // [V][2]: scaled residual, domain mask
    float* output() { return out_; }  // [V]

    cudaError_t forward(cudaStream_t s);
    // out -> gout for L = sum m (out - t)^2 / sum m t^2; sums kept on the device.
    cudaError_t loss_and_grad(const float* target, const float* mask, cudaStream_t s);
    cudaError_t backward(cudaStream_t s);  // needs forward + loss_and_grad first
    cudaError_t adam(float lr, cudaStream_t s);
    cudaError_t read_loss(double* loss, cudaStream_t s);
    cudaError_t check_error(bool* timed_out, cudaStream_t s);

    cudaError_t set_weights(const float* host, cudaStream_t s);
    cudaError_t get_weights(float* host, cudaStream_t s);
    cudaError_t get_gradients(float* host, cudaStream_t s);
    int64_t launches() const { return launches_; }

   private:
    template <class T>
    T* alloc(size_t n);
    void release();
    void pack(cudaStream_t s);
    cudaError_t tc(int l, int epi, const ConvGrid& g, ConvSrc s1, ConvSrc s2, void* out, cudaStream_t s);
    cudaError_t tc_dx(int l, const ConvGrid& g, float* gin, cudaStream_t s);
    void mask(const float* gr, const __nv_bfloat16* a, long n, cudaStream_t s);

    std::vector<void*> allocs_;
    ConvGrid g1_{}, g2_{}, g3_{};
    long V1_ = 0;
    size_t nparam_ = 0;
    size_t off_[kUNetNumLayers] = {};
    float *w_ = nullptr, *gw_ = nullptr, *m_ = nullptr, *v_ = nullptr;
    __nv_bfloat16 *wf_all_ = nullptr, *wt_all_ = nullptr;
    __nv_bfloat16* wf_[kUNetNumLayers] = {};
    __nv_bfloat16* wt_[kUNetNumLayers] = {};
    float* in_ = nullptr;
    __nv_bfloat16* a_[11] = {};
    __nv_bfloat16 *p1_ = nullptr, *p2_ = nullptr;
    float* out_ = nullptr;
    float *gA_ = nullptr, *gB_ = nullptr, *gC_ = nullptr, *gskip1_ = nullptr, *gskip2_ = nullptr, *gout_ = nullptr;
    __nv_bfloat16* hb_ = nullptr;
    double* sums_ = nullptr;
    int* err_ = nullptr;
    int adam_t_ = 0;
    int64_t launches_ = 0;
};

}  // namespace pgd
