// unet_ref.cpp -- CPU reference of the learned warm-start U-Net.
//
// TEST INFRASTRUCTURE ONLY.  The same network as the library's
// picfoam_gb300/csrc/unet.cu (3 levels, 16/32/64 channels, 3x3x3 "same"
// convolutions with zero padding, no biases, ReLU, 2x2x2 average pooling,
// nearest upsampling, skip concatenation [up(coarse), skip]) evaluated in
// FP64 with plain loops, forward and backward, as the checker of the GPU's
// forward output and weight gradients.  With emulate = 1 every value the GPU
// stores in BF16 (activations, tensor-core weights, the masked output
// gradients fed to the tensor-core input-gradient convolutions) is rounded to
// BF16 at the same place, so the two differ only by accumulation order.
// With emulate = 0 the reference is exact FP64 and is itself checked against
// finite differences.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

struct LayerDef {
    int cin, cout;
};
constexpr int kLayers = 11;
const LayerDef kDefs[kLayers] = {{2, 16},  {16, 16}, {16, 32}, {32, 32}, {32, 64}, {64, 64},
                                 {96, 32}, {32, 32}, {48, 16}, {16, 16}, {16, 1}};

double bf16(double x) {
    float f = float(x);
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

struct Grid {
    int X, Y, Z;
    long V() const { return long(X) * Y * Z; }
};

using Vec = std::vector<double>;

// tap t = (dz+1)*9 + (dy+1)*3 + (dx+1); sign -1 mirrors the offset
bool nb(const Grid& g, long v, int t, int sign, long* out) {
    const int x = int(v % g.X), y = int((v / g.X) % g.Y), z = int(v / (long(g.X) * g.Y));
    const int xn = x + sign * (t % 3 - 1), yn = y + sign * ((t / 3) % 3 - 1), zn = z + sign * (t / 9 - 1);
    if (xn < 0 || xn >= g.X || yn < 0 || yn >= g.Y || zn < 0 || zn >= g.Z) return false;
    *out = (long(zn) * g.Y + yn) * g.X + xn;
    return true;
}

// y[v][co] = sum_t sum_ci x[v + d_t][ci] w[t][co][ci]
Vec conv(const Grid& g, const Vec& x, int ci, int co, const Vec& w) {
    Vec y(size_t(g.V()) * co, 0.0);
    for (long v = 0; v < g.V(); ++v)
        for (int t = 0; t < 27; ++t) {
            long n;
            if (!nb(g, v, t, 1, &n)) continue;
            for (int o = 0; o < co; ++o) {
                double s = 0.0;
                for (int i = 0; i < ci; ++i) s += x[n * ci + i] * w[(size_t(t) * co + o) * ci + i];
                y[v * co + o] += s;
            }
        }
    return y;
}

// g_x[u][ci] = sum_t sum_co h[u - d_t][co] w[t][co][ci]
Vec conv_dx(const Grid& g, const Vec& h, int ci, int co, const Vec& w) {
    Vec gx(size_t(g.V()) * ci, 0.0);
    for (long u = 0; u < g.V(); ++u)
        for (int t = 0; t < 27; ++t) {
            long n;
            if (!nb(g, u, t, -1, &n)) continue;
            for (int i = 0; i < ci; ++i) {
                double s = 0.0;
                for (int o = 0; o < co; ++o) s += h[n * co + o] * w[(size_t(t) * co + o) * ci + i];
                gx[u * ci + i] += s;
            }
        }
    return gx;
}

// dW[t][co][ci] = sum_v h[v][co] x[v + d_t][ci]
void conv_dw(const Grid& g, const Vec& h, const Vec& x, int ci, int co, double* dw) {
    for (long v = 0; v < g.V(); ++v)
        for (int t = 0; t < 27; ++t) {
            long n;
            if (!nb(g, v, t, 1, &n)) continue;
            for (int o = 0; o < co; ++o) {
                const double hv = h[v * co + o];
                if (hv == 0.0) continue;
                for (int i = 0; i < ci; ++i) dw[(size_t(t) * co + o) * ci + i] += hv * x[n * ci + i];
            }
        }
}

Vec relu(Vec a, bool em) {
    for (double& x : a) x = x > 0 ? (em ? bf16(x) : x) : 0.0;
    return a;
}

Vec pool(const Grid& g, const Vec& a, int C, bool em) {
    const Grid h{g.X / 2, g.Y / 2, g.Z / 2};
    Vec p(size_t(h.V()) * C, 0.0);
    for (long vc = 0; vc < h.V(); ++vc) {
        const int x = int(vc % h.X), y = int((vc / h.X) % h.Y), z = int(vc / (long(h.X) * h.Y));
        for (int k = 0; k < 8; ++k) {
            const long vf = (long(2 * z + (k >> 2)) * g.Y + 2 * y + ((k >> 1) & 1)) * g.X + 2 * x + (k & 1);
            for (int c = 0; c < C; ++c) p[vc * C + c] += a[vf * C + c];
        }
        for (int c = 0; c < C; ++c) p[vc * C + c] = em ? bf16(0.125 * p[vc * C + c]) : 0.125 * p[vc * C + c];
    }
    return p;
}

long parent(const Grid& g, long v) {
    const int x = int(v % g.X), y = int((v / g.X) % g.Y), z = int(v / (long(g.X) * g.Y));
    return (long(z >> 1) * (g.Y >> 1) + (y >> 1)) * (g.X >> 1) + (x >> 1);
}

// [up(coarse), skip] at the fine grid g
Vec upcat(const Grid& g, const Vec& coarse, int C1, const Vec& skip, int C2) {
    Vec o(size_t(g.V()) * (C1 + C2));
    for (long v = 0; v < g.V(); ++v) {
        const long p = parent(g, v);
        for (int c = 0; c < C1; ++c) o[v * (C1 + C2) + c] = coarse[p * C1 + c];
        for (int c = 0; c < C2; ++c) o[v * (C1 + C2) + C1 + c] = skip[v * C2 + c];
    }
    return o;
}

struct Net {
    Grid g1, g2, g3;
    bool em;
    std::vector<Vec> w;   // per layer, as used (BF16-rounded for tensor-core layers when em)
    Vec in, a1, a2, p1, a3, a4, p2, a5, a6, cat2, a7, a8, cat1, a9, a10, out;

    Net(int X, int Y, int Z, const float* wf, bool emulate) : g1{X, Y, Z}, g2{X / 2, Y / 2, Z / 2},
                                                           g3{X / 4, Y / 4, Z / 4}, em(emulate) {
        size_t off = 0;
        for (int l = 0; l < kLayers; ++l) {
            const size_t n = size_t(27) * kDefs[l].cin * kDefs[l].cout;
            Vec v(n);
            const bool tc = l >= 1 && l <= 9;
            for (size_t i = 0; i < n; ++i) v[i] = (em && tc) ? bf16(wf[off + i]) : double(wf[off + i]);
            w.push_back(v);
            off += n;
        }
    }

    void forward(const float* x) {
        in.assign(x, x + 2 * g1.V());
        a1 = relu(conv(g1, in, 2, 16, w[0]), em);
        a2 = relu(conv(g1, a1, 16, 16, w[1]), em);
        p1 = pool(g1, a2, 16, em);
        a3 = relu(conv(g2, p1, 16, 32, w[2]), em);
        a4 = relu(conv(g2, a3, 32, 32, w[3]), em);
        p2 = pool(g2, a4, 32, em);
        a5 = relu(conv(g3, p2, 32, 64, w[4]), em);
        a6 = relu(conv(g3, a5, 64, 64, w[5]), em);
        cat2 = upcat(g2, a6, 64, a4, 32);
        a7 = relu(conv(g2, cat2, 96, 32, w[6]), em);
        a8 = relu(conv(g2, a7, 32, 32, w[7]), em);
        cat1 = upcat(g1, a8, 32, a2, 16);
        a9 = relu(conv(g1, cat1, 48, 16, w[8]), em);
        a10 = relu(conv(g1, a9, 16, 16, w[9]), em);
        out = conv(g1, a10, 16, 1, w[10]);
    }

    // masked output gradient, BF16-rounded when emulating
    Vec masked(const Vec& gr, const Vec& a) const {
        Vec h(gr.size());
        for (size_t i = 0; i < gr.size(); ++i) h[i] = a[i] > 0 ? (em ? bf16(gr[i]) : gr[i]) : 0.0;
        return h;
    }

    double backward(const float* target, const float* mask, double* grad) {
        const long V = g1.V();
        double num = 0.0, den = 0.0;
        for (long v = 0; v < V; ++v) {
            const double d = out[v] - target[v];
            num += mask[v] * d * d;
            den += mask[v] * double(target[v]) * target[v];
        }
        if (!(den > 0)) den = 1.0;
        Vec gout(V);
        for (long v = 0; v < V; ++v) gout[v] = 2.0 * mask[v] * (out[v] - target[v]) / den;
        std::vector<double*> gw(kLayers);
        size_t off = 0;
        for (int l = 0; l < kLayers; ++l) {
            gw[l] = grad + off;
            off += size_t(27) * kDefs[l].cin * kDefs[l].cout;
        }
        std::fill(grad, grad + off, 0.0);
        conv_dw(g1, gout, a10, 16, 1, gw[10]);
        Vec ga10 = conv_dx(g1, gout, 16, 1, w[10]);
        Vec h = masked(ga10, a10);
        conv_dw(g1, h, a9, 16, 16, gw[9]);
        Vec ga9 = conv_dx(g1, h, 16, 16, w[9]);
        h = masked(ga9, a9);
        conv_dw(g1, h, cat1, 48, 16, gw[8]);
        Vec gcat1 = conv_dx(g1, h, 48, 16, w[8]);
        Vec ga2(size_t(V) * 16, 0.0), ga8(size_t(g2.V()) * 32, 0.0);
        for (long v = 0; v < V; ++v) {
            const long p = parent(g1, v);
            for (int c = 0; c < 32; ++c) ga8[p * 32 + c] += gcat1[v * 48 + c];
            for (int c = 0; c < 16; ++c) ga2[v * 16 + c] += gcat1[v * 48 + 32 + c];
        }
        h = masked(ga8, a8);
        conv_dw(g2, h, a7, 32, 32, gw[7]);
        Vec ga7 = conv_dx(g2, h, 32, 32, w[7]);
        h = masked(ga7, a7);
        conv_dw(g2, h, cat2, 96, 32, gw[6]);
        Vec gcat2 = conv_dx(g2, h, 96, 32, w[6]);
        Vec ga4(size_t(g2.V()) * 32, 0.0), ga6(size_t(g3.V()) * 64, 0.0);
        for (long v = 0; v < g2.V(); ++v) {
            const long p = parent(g2, v);
            for (int c = 0; c < 64; ++c) ga6[p * 64 + c] += gcat2[v * 96 + c];
            for (int c = 0; c < 32; ++c) ga4[v * 32 + c] += gcat2[v * 96 + 64 + c];
        }
        h = masked(ga6, a6);
        conv_dw(g3, h, a5, 64, 64, gw[5]);
        Vec ga5 = conv_dx(g3, h, 64, 64, w[5]);
        h = masked(ga5, a5);
        conv_dw(g3, h, p2, 32, 64, gw[4]);
        Vec gp2 = conv_dx(g3, h, 32, 64, w[4]);
        for (long v = 0; v < g2.V(); ++v) {
            const long p = parent(g2, v);
            for (int c = 0; c < 32; ++c) ga4[v * 32 + c] += 0.125 * gp2[p * 32 + c];
        }
        h = masked(ga4, a4);
        conv_dw(g2, h, a3, 32, 32, gw[3]);
        Vec ga3 = conv_dx(g2, h, 32, 32, w[3]);
        h = masked(ga3, a3);
        conv_dw(g2, h, p1, 16, 32, gw[2]);
        Vec gp1 = conv_dx(g2, h, 16, 32, w[2]);
        for (long v = 0; v < V; ++v) {
            const long p = parent(g1, v);
            for (int c = 0; c < 16; ++c) ga2[v * 16 + c] += 0.125 * gp1[p * 16 + c];
        }
        h = masked(ga2, a2);
        conv_dw(g1, h, a1, 16, 16, gw[1]);
        Vec ga1 = conv_dx(g1, h, 16, 16, w[1]);
        h = masked(ga1, a1);
        conv_dw(g1, h, in, 2, 16, gw[0]);
        return num / den;
    }
};

bool grid_ok(int X, int Y, int Z) { return X > 0 && Y > 0 && Z > 0 && X % 4 == 0 && Y % 4 == 0 && Z % 4 == 0; }

}  // namespace

extern "C" {

size_t oracle_unet_param_count(void) {
    size_t n = 0;
    for (int l = 0; l < kLayers; ++l) n += size_t(27) * kDefs[l].cin * kDefs[l].cout;
    return n;
}

int oracle_unet_forward(int X, int Y, int Z, const float* w, const float* in, int emulate, double* out) {
    if (!grid_ok(X, Y, Z) || !w || !in || !out) return PICGPU_INVALID_ARG;
    Net n(X, Y, Z, w, emulate != 0);
    n.forward(in);
    std::memcpy(out, n.out.data(), n.out.size() * sizeof(double));
    return 0;
}

int oracle_unet_gradients(int X, int Y, int Z, const float* w, const float* in, const float* target,
                          const float* mask, int emulate, double* grad, double* loss) {
    if (!grid_ok(X, Y, Z) || !w || !in || !target || !mask || !grad) return PICGPU_INVALID_ARG;
    Net n(X, Y, Z, w, emulate != 0);
    n.forward(in);
    const double l = n.backward(target, mask, grad);
    if (loss) *loss = l;
    return 0;
}

}  // extern "C"
