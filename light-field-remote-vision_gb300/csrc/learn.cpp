// learn.cpp -- the learned warm start: a 4-scale encoder-decoder whose every convolution runs on the tcgen05
// implicit-GEMM kernels (kernels_learn.cu), its training step (backward + Adam) and inference.
//
// Network (input kNetIn = 48 channels at H x W, H and W multiples of 8; ~1.23 M parameters):
//   e0 = relu(conv3x3(in, 48->32))            H      e1 = relu(conv3x3/2(e0, 32->64))     H/2
//   e2 = relu(conv3x3/2(e1, 64->128))         H/4    e3 = relu(conv3x3/2(e2, 128->256))   H/8
//   b  = relu(conv3x3(e3, 256->256))          H/8
//   s5 = relu(up2(conv1x1(b, 256->128)) + e2) H/4    d6 = relu(conv3x3(s5, 128->128))     H/4
//   s7 = relu(up2(conv1x1(d6, 128->64)) + e1) H/2    d8 = relu(conv3x3(s7, 64->64))       H/2
//   s9 = relu(up2(conv1x1(d8, 64->32)) + e0)  H      d10 = relu(conv3x3(s9, 32->32))      H
//   y  = conv3x3(d10, 32->3)                  H      prediction = u0 + y (u0: the solver's anchor)
// Activations and weights are BF16, accumulation FP32 (TMEM), master weights and Adam state FP32.
// Parameters, flat FP32: per layer W[cout][tap][cin] (tap = 3 ky + kx) then bias[cout].
#include "context.h"
#include "kernels.h"
#include "lfrv.h"
#include "lfrv_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace lfrv {

namespace {

struct LayerDef {
    int cin, cout, ks, stride, relu;
};
constexpr int kLayers = 12;
constexpr LayerDef kNet[kLayers] = {
    {48, 32, 3, 1, 1},   {32, 64, 3, 2, 1},  {64, 128, 3, 2, 1}, {128, 256, 3, 2, 1},
    {256, 256, 3, 1, 1}, {256, 128, 1, 1, 0}, {128, 128, 3, 1, 1}, {128, 64, 1, 1, 0},
    {64, 64, 3, 1, 1},   {64, 32, 1, 1, 0},  {32, 32, 3, 1, 1},   {32, 3, 3, 1, 0},
};
static_assert(kNet[0].cin == kLearnChannels, "network input width");

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// Tensors of one forward/backward pass: channels and pyramid level (size H >> level x W >> level).
enum Tensor {
    A0, A1, A2, A3, A4, T5, S5, A6, T7, S7, A8, T9, S9, A10,                   // forward (BF16)
    DY11, G10, GS9, DT9, G8, GS7, DT7, G6, GS5, DT5, G4, G3, G2, G1, G0, kTensors  // backward (BF16)
};
constexpr int kTensorC[kTensors] = {32, 64, 128, 256, 256, 128, 128, 128, 64, 64, 64, 32, 32, 32,
                                    16, 32, 32, 32, 64, 64, 64, 128, 128, 128, 256, 256, 128, 64, 32};
constexpr int kTensorL[kTensors] = {0, 1, 2, 3, 3, 3, 2, 2, 2, 1, 1, 1, 0, 0,
                                    0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 1, 0};

struct Layer {
    LayerDef d;
    int cst, taps, Kf, Kpad, Kd, Kdpad;
    size_t w_off, b_off;
    DevBuf Wb, Wt;
};

// splitmix64 and Box-Muller: the seeded initial weights.
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace

}  // namespace lfrv

struct lfrv_warmstart {
    lfrv_ctx *ctx = nullptr;
    lfrv::Layer L[lfrv::kLayers];
    size_t nparams = 0;
    lfrv::DevBuf params, grads, adam_m, adam_v;
    long long step = 0;
    int batch = 0, H = 0, W = 0;
    lfrv::DevBuf t[lfrv::kTensors];
    lfrv::DevBuf y, partial, bias_part, loss_part, err;
};

namespace lfrv {

namespace {

constexpr int kBiasBlocks = 152;
constexpr int kLossBlocks = 304;
constexpr size_t kParamSlack = 256;  // zeros after the last bias: the padded output head reads 16 bias values

void net_check(lfrv_warmstart *net) {
    if (!net || !net->ctx) raise(LFRV_E_ARG, "null warm-start network");
}

void net_layout(lfrv_warmstart *net) {
    size_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
        Layer &L = net->L[l];
        L.d = kNet[l];
        L.cst = std::max(16, L.d.cout);
        L.taps = L.d.ks * L.d.ks;
        L.Kf = L.taps * L.d.cin;
        L.Kpad = round_up(L.Kf, 64);
        L.Kd = L.taps * L.cst;
        L.Kdpad = round_up(L.Kd, 64);
        L.w_off = off;
        off += (size_t)L.d.cout * L.Kf;
        L.b_off = off;
        off += (size_t)L.d.cout;
        L.Wb.ensure((size_t)L.cst * L.Kpad * 2);
        L.Wt.ensure((size_t)L.d.cin * L.Kdpad * 2);
    }
    net->nparams = off;
}

// BF16 GEMM copies of the FP32 master weights.
void net_pack(lfrv_warmstart *net) {
    lfrv_ctx *c = net->ctx;
    for (int l = 0; l < kLayers; ++l) {
        Layer &L = net->L[l];
        LFRV_CUDA(launch_pack_weights(L.d.cout, L.cst, L.d.cin, L.taps, L.Kpad, L.Kdpad,
                                      net->params.as<float>() + L.w_off, L.Wb.p, L.Wt.p, c->stream, c->launches));
    }
}

void net_init_params(lfrv_warmstart *net, unsigned long long seed) {
    std::vector<float> h(net->nparams + kParamSlack, 0.f);
    Rng rng{seed ^ 0x6C6672765F776172ull};
    for (int l = 0; l < kLayers; ++l) {
        const Layer &L = net->L[l];
        // He initialisation for ReLU layers, LeCun for the linear ones; the output layer starts at zero, so the
        // untrained prediction is the anchor itself
        double sd = std::sqrt((L.d.relu ? 2.0 : 1.0) / (double)L.Kf);
        if (l == kLayers - 1) sd = 0.0;
        for (size_t i = 0; i < (size_t)L.d.cout * L.Kf; ++i) h[L.w_off + i] = (float)(sd * rng.normal());
    }
    LFRV_CUDA(cudaMemcpyAsync(net->params.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice,
                              net->ctx->stream));
    LFRV_CUDA(cudaMemsetAsync(net->adam_m.p, 0, net->nparams * sizeof(float), net->ctx->stream));
    LFRV_CUDA(cudaMemsetAsync(net->adam_v.p, 0, net->nparams * sizeof(float), net->ctx->stream));
    net->step = 0;
    net_pack(net);
}

void net_shape(lfrv_warmstart *net, int batch, int H, int W) {
    if (batch < 1 || H < 8 || W < 8 || H % 8 || W % 8)
        raise(LFRV_E_ARG, "warm-start network: batch >= 1 and H, W multiples of 8 (got %d x %d x %d)", batch, H, W);
    if ((size_t)batch * H * W > ((size_t)1 << 30)) raise(LFRV_E_ARG, "warm-start network: batch too large");
    if (batch == net->batch && H == net->H && W == net->W) return;
    for (int i = 0; i < kTensors; ++i) {
        const size_t px = (size_t)batch * (H >> kTensorL[i]) * (W >> kTensorL[i]);
        net->t[i].ensure(px * kTensorC[i] * 2);
    }
    net->y.ensure((size_t)batch * H * W * 16 * sizeof(float));
    net->batch = batch;
    net->H = H;
    net->W = W;
}

int *net_err(lfrv_warmstart *net) { return net->err.as<int>(); }

// Forward of layer l (input at `level`); with upskip, outb receives relu(up2(conv) + upskip) at level - 1.
void conv_forward(lfrv_warmstart *net, int l, const void *x, int level, void *outb, float *outf,
                  const void *upskip = nullptr) {
    const Layer &L = net->L[l];
    const int Hin = net->H >> level, Win = net->W >> level;
    ConvGemm g{};
    g.src = x;
    g.C = L.d.cin;
    g.Hs = Hin;
    g.Ws = Win;
    g.batch = net->batch;
    g.Ho = Hin / L.d.stride;
    g.Wo = Win / L.d.stride;
    g.ks = L.d.ks;
    g.stride = L.d.stride;
    g.dgrad = 0;
    g.K = L.Kf;
    g.wt = L.Wb.p;
    g.ldw = L.Kpad;
    g.N = L.cst;
    g.bias = net->params.as<float>() + L.b_off;
    g.relu = L.d.relu;
    g.outb = outb;
    g.outf = outf;
    g.upskip = upskip;
    LFRV_CUDA(launch_conv_tc(g, net_err(net), net->ctx->stream, net->ctx->launches));
}

// dX of layer l (input at `level`) from dY, + add, zeroed where mask <= 0.
void conv_dgrad(lfrv_warmstart *net, int l, const void *dy, int level, const void *add, const void *mask, void *dx) {
    const Layer &L = net->L[l];
    const int Hin = net->H >> level, Win = net->W >> level;
    ConvGemm g{};
    g.src = dy;
    g.C = L.cst;
    g.Hs = Hin / L.d.stride;
    g.Ws = Win / L.d.stride;
    g.batch = net->batch;
    g.Ho = Hin;
    g.Wo = Win;
    g.ks = L.d.ks;
    g.stride = L.d.stride;
    g.dgrad = 1;
    g.K = L.Kd;
    g.wt = L.Wt.p;
    g.ldw = L.Kdpad;
    g.N = L.d.cin;
    g.add = add;
    g.mask = mask;
    g.outb = dx;
    LFRV_CUDA(launch_conv_tc(g, net_err(net), net->ctx->stream, net->ctx->launches));
}

// dW and db of layer l (input x at `level`, output gradient dy) into the flat gradient.
void conv_wgrad(lfrv_warmstart *net, int l, const void *x, int level, const void *dy) {
    const Layer &L = net->L[l];
    lfrv_ctx *c = net->ctx;
    const int Hin = net->H >> level, Win = net->W >> level;
    WgradGemm g{};
    g.x = x;
    g.Cin = L.d.cin;
    g.Hx = Hin;
    g.Wx = Win;
    g.dy = dy;
    g.Cout = L.cst;
    g.Ho = Hin / L.d.stride;
    g.Wo = Win / L.d.stride;
    g.batch = net->batch;
    g.ks = L.d.ks;
    g.stride = L.d.stride;
    g.Kf = L.Kf;
    g.Mpad = round_up(L.Kf, 128);
    const int P = net->batch * g.Ho * g.Wo;
    const int mt = g.Mpad / 128, max_splits = (P + 63) / 64;
    int splits = std::min(max_splits, std::max(1, (2 * 152 + mt - 1) / mt));
    g.chunk = round_up((P + splits - 1) / splits, 64);
    splits = (P + g.chunk - 1) / g.chunk;
    net->partial.ensure((size_t)splits * g.Mpad * L.cst * sizeof(float));
    g.partial = net->partial.as<float>();
    float *grad = net->grads.as<float>();
    LFRV_CUDA(launch_wgrad_tc(g, splits, L.d.cout, grad + L.w_off, net_err(net), c->stream, c->launches));
    LFRV_CUDA(launch_bias_grad(P, L.cst, L.d.cout, dy, net->bias_part.as<float>(), kBiasBlocks, grad + L.b_off,
                               c->stream, c->launches));
}

void forward(lfrv_warmstart *net, const void *in) {
    lfrv_ctx *c = net->ctx;
    auto b = [&](int i) { return net->t[i].p; };
    conv_forward(net, 0, in, 0, b(A0), nullptr);
    conv_forward(net, 1, b(A0), 0, b(A1), nullptr);
    conv_forward(net, 2, b(A1), 1, b(A2), nullptr);
    conv_forward(net, 3, b(A2), 2, b(A3), nullptr);
    conv_forward(net, 4, b(A3), 3, b(A4), nullptr);
    // decoder: the 1 x 1 convolution's epilogue upsamples, adds the skip and applies the ReLU (s = relu(up2(t) + e))
    conv_forward(net, 5, b(A4), 3, b(S5), nullptr, b(A2));
    conv_forward(net, 6, b(S5), 2, b(A6), nullptr);
    conv_forward(net, 7, b(A6), 2, b(S7), nullptr, b(A1));
    conv_forward(net, 8, b(S7), 1, b(A8), nullptr);
    conv_forward(net, 9, b(A8), 1, b(S9), nullptr, b(A0));
    conv_forward(net, 10, b(S9), 0, b(A10), nullptr);
    conv_forward(net, 11, b(A10), 0, nullptr, net->y.as<float>());
}

void backward(lfrv_warmstart *net, const void *in) {
    lfrv_ctx *c = net->ctx;
    auto b = [&](int i) { return net->t[i].p; };
    const int B = net->batch, H = net->H, W = net->W;
    conv_wgrad(net, 11, b(A10), 0, b(DY11));
    conv_dgrad(net, 11, b(DY11), 0, nullptr, b(A10), b(G10));
    conv_wgrad(net, 10, b(S9), 0, b(G10));
    conv_dgrad(net, 10, b(G10), 0, nullptr, b(S9), b(GS9));
    LFRV_CUDA(launch_down_sum(B, H >> 1, W >> 1, 32, b(GS9), b(DT9), c->stream, c->launches));
    conv_wgrad(net, 9, b(A8), 1, b(DT9));
    conv_dgrad(net, 9, b(DT9), 1, nullptr, b(A8), b(G8));
    conv_wgrad(net, 8, b(S7), 1, b(G8));
    conv_dgrad(net, 8, b(G8), 1, nullptr, b(S7), b(GS7));
    LFRV_CUDA(launch_down_sum(B, H >> 2, W >> 2, 64, b(GS7), b(DT7), c->stream, c->launches));
    conv_wgrad(net, 7, b(A6), 2, b(DT7));
    conv_dgrad(net, 7, b(DT7), 2, nullptr, b(A6), b(G6));
    conv_wgrad(net, 6, b(S5), 2, b(G6));
    conv_dgrad(net, 6, b(G6), 2, nullptr, b(S5), b(GS5));
    LFRV_CUDA(launch_down_sum(B, H >> 3, W >> 3, 128, b(GS5), b(DT5), c->stream, c->launches));
    conv_wgrad(net, 5, b(A4), 3, b(DT5));
    conv_dgrad(net, 5, b(DT5), 3, nullptr, b(A4), b(G4));
    conv_wgrad(net, 4, b(A3), 3, b(G4));
    conv_dgrad(net, 4, b(G4), 3, nullptr, b(A3), b(G3));
    conv_wgrad(net, 3, b(A2), 2, b(G3));
    conv_dgrad(net, 3, b(G3), 2, b(GS5), b(A2), b(G2));
    conv_wgrad(net, 2, b(A1), 1, b(G2));
    conv_dgrad(net, 2, b(G2), 1, b(GS7), b(A1), b(G1));
    conv_wgrad(net, 1, b(A0), 0, b(G1));
    conv_dgrad(net, 1, b(G1), 0, b(GS9), b(A0), b(G0));
    conv_wgrad(net, 0, in, 0, b(G0));
}

// Output head: prediction and/or the loss partials + dY of the last layer (asynchronous).
void head(lfrv_warmstart *net, const float *u0, const float *target, float *pred) {
    lfrv_ctx *c = net->ctx;
    LFRV_CUDA(launch_output_head(net->batch, net->H * net->W, 16, net->y.as<float>(), u0, target, pred,
                                 target ? net->t[DY11].p : nullptr, net->loss_part.as<double>(), kLossBlocks,
                                 c->stream, c->launches));
}

double read_loss_and_check(lfrv_warmstart *net) {
    lfrv_ctx *c = net->ctx;
    std::vector<double> lp(kLossBlocks);
    int err = 0;
    LFRV_CUDA(cudaMemcpyAsync(lp.data(), net->loss_part.p, kLossBlocks * sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    LFRV_CUDA(cudaMemcpyAsync(&err, net->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LFRV_CUDA(cudaStreamSynchronize(c->stream));
    if (err) {
        LFRV_CUDA(cudaMemsetAsync(net->err.p, 0, sizeof(int), c->stream));
        raise(LFRV_E_TIMEOUT, "tensor-core convolution: an mbarrier wait gave up");
    }
    double s = 0.0;
    for (double v : lp) s += v;
    return s / (3.0 * net->batch * (double)net->H * net->W);
}

void check_err(lfrv_warmstart *net) {
    int err = 0;
    LFRV_CUDA(cudaMemcpyAsync(&err, net->err.p, sizeof(int), cudaMemcpyDeviceToHost, net->ctx->stream));
    LFRV_CUDA(cudaStreamSynchronize(net->ctx->stream));
    if (err) {
        LFRV_CUDA(cudaMemsetAsync(net->err.p, 0, sizeof(int), net->ctx->stream));
        raise(LFRV_E_TIMEOUT, "tensor-core convolution: an mbarrier wait gave up");
    }
}

void adam(lfrv_warmstart *net, float lr) {
    const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
    net->step += 1;
    const double c1 = 1.0 - std::pow(b1, (double)net->step), c2 = 1.0 - std::pow(b2, (double)net->step);
    const float lr_t = (float)(lr * std::sqrt(c2) / c1), eps_t = (float)(eps * std::sqrt(c2));
    LFRV_CUDA(launch_adam(net->nparams, net->params.as<float>(), net->grads.as<float>(), net->adam_m.as<float>(),
                          net->adam_v.as<float>(), lr_t, (float)b1, (float)b2, eps_t, net->ctx->stream,
                          net->ctx->launches));
    net_pack(net);
}

}  // namespace

// Internal entry for the solver paths: prediction = u0 + net(input) for one image (asynchronous, no checks).
void warmstart_predict_async(lfrv_warmstart *net, int H, int W, const void *d_input, const float *d_u0, float *d_pred) {
    net_shape(net, 1, H, W);
    forward(net, d_input);
    head(net, d_u0, nullptr, d_pred);
}

void warmstart_check(lfrv_warmstart *net) { check_err(net); }

lfrv_ctx *warmstart_ctx(lfrv_warmstart *net) { return net ? net->ctx : nullptr; }

// Single convolution through the tensor-core kernels (tests of the GEMM paths in isolation). mode 0: forward
// out[b][y][x][co]; 1: data gradient out[b][y][x][ci] of the input; 2: weight gradient out[co][tap][ci].
static void conv_single(lfrv_ctx *c, int mode, int batch, int Hin, int Win, int Cin, int Cout, int ks, int stride,
                        const void *x, const void *dy, const float *w, float *out) {
    if ((ks != 1 && ks != 3) || (stride != 1 && stride != 2) || Cin % 8 || Cin < 8 || batch < 1 || Hin < 1 ||
        Win < 1 || Hin % stride || Win % stride)
        raise(LFRV_E_ARG, "conv: unsupported geometry");
    if (Cout != 16 && Cout != 32 && Cout != 64 && Cout != 128 && Cout != 256)
        raise(LFRV_E_ARG, "conv: Cout must be 16, 32, 64, 128 or 256");
    if (mode == 1 && Cin != 16 && Cin != 32 && Cin != 64 && Cin != 128 && Cin != 256)
        raise(LFRV_E_ARG, "conv: the data gradient needs Cin of 16, 32, 64, 128 or 256");
    const int taps = ks * ks, Kf = taps * Cin, Kpad = round_up(Kf, 64), Kd = taps * Cout, Kdpad = round_up(Kd, 64);
    DevBuf wf, Wb, Wt, err, part;
    wf.ensure((size_t)Cout * Kf * sizeof(float));
    Wb.ensure((size_t)Cout * Kpad * 2);
    Wt.ensure((size_t)Cin * Kdpad * 2);
    err.ensure(sizeof(int));
    LFRV_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c->stream));
    LFRV_CUDA(cudaMemcpyAsync(wf.p, w, (size_t)Cout * Kf * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    LFRV_CUDA(launch_pack_weights(Cout, Cout, Cin, taps, Kpad, Kdpad, wf.as<float>(), Wb.p, Wt.p, c->stream,
                                  c->launches));
    const int Ho = Hin / stride, Wo = Win / stride;
    if (mode == 0 || mode == 1) {
        ConvGemm g{};
        g.batch = batch;
        g.ks = ks;
        g.stride = stride;
        g.outf = out;
        if (mode == 0) {
            g.src = x;
            g.C = Cin;
            g.Hs = Hin;
            g.Ws = Win;
            g.Ho = Ho;
            g.Wo = Wo;
            g.K = Kf;
            g.wt = Wb.p;
            g.ldw = Kpad;
            g.N = Cout;
        } else {
            g.src = dy;
            g.C = Cout;
            g.Hs = Ho;
            g.Ws = Wo;
            g.Ho = Hin;
            g.Wo = Win;
            g.dgrad = 1;
            g.K = Kd;
            g.wt = Wt.p;
            g.ldw = Kdpad;
            g.N = Cin;
        }
        LFRV_CUDA(launch_conv_tc(g, err.as<int>(), c->stream, c->launches));
    } else {
        WgradGemm g{};
        g.x = x;
        g.Cin = Cin;
        g.Hx = Hin;
        g.Wx = Win;
        g.dy = dy;
        g.Cout = Cout;
        g.Ho = Ho;
        g.Wo = Wo;
        g.batch = batch;
        g.ks = ks;
        g.stride = stride;
        g.Kf = Kf;
        g.Mpad = round_up(Kf, 128);
        const int P = batch * Ho * Wo;
        int splits = std::min((P + 63) / 64, std::max(1, (2 * 152 + g.Mpad / 128 - 1) / (g.Mpad / 128)));
        g.chunk = round_up((P + splits - 1) / splits, 64);
        splits = (P + g.chunk - 1) / g.chunk;
        part.ensure((size_t)splits * g.Mpad * Cout * sizeof(float));
        g.partial = part.as<float>();
        LFRV_CUDA(launch_wgrad_tc(g, splits, Cout, out, err.as<int>(), c->stream, c->launches));
    }
    int e = 0;
    LFRV_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LFRV_CUDA(cudaStreamSynchronize(c->stream));
    if (e) raise(LFRV_E_TIMEOUT, "tensor-core convolution: an mbarrier wait gave up");
}

}  // namespace lfrv

using namespace lfrv;

extern "C" long long lfrv_warmstart_param_count(void) {
    long long n = 0;
    for (int l = 0; l < kLayers; ++l) n += (long long)kNet[l].cout * (kNet[l].ks * kNet[l].ks * kNet[l].cin + 1);
    return n;
}

extern "C" int lfrv_warmstart_create(lfrv_ctx *ctx, unsigned long long seed, lfrv_warmstart **out) {
    LFRV_API_BEGIN
    if (!ctx || !out) raise(LFRV_E_ARG, "null argument");
    *out = nullptr;
    lfrv_warmstart *net = new lfrv_warmstart();
    try {
        net->ctx = ctx;
        LFRV_CUDA(cudaSetDevice(ctx->device));
        net_layout(net);
        net->params.ensure((net->nparams + kParamSlack) * sizeof(float));
        net->grads.ensure(net->nparams * sizeof(float));
        net->adam_m.ensure(net->nparams * sizeof(float));
        net->adam_v.ensure(net->nparams * sizeof(float));
        net->bias_part.ensure((size_t)kBiasBlocks * 256 * sizeof(float));
        net->loss_part.ensure(kLossBlocks * sizeof(double));
        net->err.ensure(sizeof(int));
        LFRV_CUDA(cudaMemsetAsync(net->err.p, 0, sizeof(int), ctx->stream));
        net_init_params(net, seed);
        LFRV_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        delete net;
        throw;
    }
    *out = net;
    LFRV_API_END
}

extern "C" void lfrv_warmstart_destroy(lfrv_warmstart *net) {
    if (!net) return;
    if (net->ctx) cudaStreamSynchronize(net->ctx->stream);
    delete net;
}

extern "C" int lfrv_warmstart_get_params(lfrv_warmstart *net, float *params) {
    LFRV_API_BEGIN
    net_check(net);
    if (!params) raise(LFRV_E_ARG, "null argument");
    LFRV_CUDA(cudaMemcpyAsync(params, net->params.p, net->nparams * sizeof(float), cudaMemcpyDeviceToHost,
                              net->ctx->stream));
    LFRV_CUDA(cudaStreamSynchronize(net->ctx->stream));
    LFRV_API_END
}

extern "C" int lfrv_warmstart_set_params(lfrv_warmstart *net, const float *params) {
    LFRV_API_BEGIN
    net_check(net);
    if (!params) raise(LFRV_E_ARG, "null argument");
    LFRV_CUDA(cudaMemcpyAsync(net->params.p, params, net->nparams * sizeof(float), cudaMemcpyHostToDevice,
                              net->ctx->stream));
    LFRV_CUDA(cudaMemsetAsync(net->adam_m.p, 0, net->nparams * sizeof(float), net->ctx->stream));
    LFRV_CUDA(cudaMemsetAsync(net->adam_v.p, 0, net->nparams * sizeof(float), net->ctx->stream));
    net->step = 0;
    net_pack(net);
    LFRV_CUDA(cudaStreamSynchronize(net->ctx->stream));
    LFRV_API_END
}

extern "C" int lfrv_warmstart_forward_dev(lfrv_warmstart *net, int batch, int H, int W, const void *d_input,
                                          const float *d_u0, float *d_pred) {
    LFRV_API_BEGIN
    net_check(net);
    if (!d_input || !d_u0 || !d_pred) raise(LFRV_E_ARG, "null argument");
    net_shape(net, batch, H, W);
    forward(net, d_input);
    head(net, d_u0, nullptr, d_pred);
    check_err(net);
    LFRV_API_END
}

extern "C" int lfrv_warmstart_gradients_dev(lfrv_warmstart *net, int batch, int H, int W, const void *d_input,
                                            const float *d_u0, const float *d_target, double *loss, float *grads) {
    LFRV_API_BEGIN
    net_check(net);
    if (!d_input || !d_u0 || !d_target) raise(LFRV_E_ARG, "null argument");
    net_shape(net, batch, H, W);
    forward(net, d_input);
    head(net, d_u0, d_target, nullptr);
    backward(net, d_input);
    const double l = read_loss_and_check(net);
    if (loss) *loss = l;
    if (grads) {
        LFRV_CUDA(cudaMemcpyAsync(grads, net->grads.p, net->nparams * sizeof(float), cudaMemcpyDeviceToHost,
                                  net->ctx->stream));
        LFRV_CUDA(cudaStreamSynchronize(net->ctx->stream));
    }
    LFRV_API_END
}

extern "C" int lfrv_warmstart_train_step_dev(lfrv_warmstart *net, int batch, int H, int W, const void *d_input,
                                             const float *d_u0, const float *d_target, float lr, double *loss) {
    LFRV_API_BEGIN
    net_check(net);
    if (!d_input || !d_u0 || !d_target || !(lr > 0.f)) raise(LFRV_E_ARG, "bad argument");
    net_shape(net, batch, H, W);
    forward(net, d_input);
    head(net, d_u0, d_target, nullptr);
    backward(net, d_input);
    adam(net, lr);
    const double l = read_loss_and_check(net);
    if (loss) *loss = l;
    LFRV_API_END
}

extern "C" int lfrv_set_conv_kernel(int which) {
    if (which < 0 || which > 2) return fail(LFRV_E_ARG, "conv kernel choice must be 0, 1 or 2 (got %d)", which);
    set_conv_kernel_pref(which);
    return LFRV_OK;
}

extern "C" int lfrv_conv_bf16_dev(lfrv_ctx *ctx, int mode, int batch, int H, int W, int Cin, int Cout, int ks,
                                  int stride, const void *d_x, const void *d_dy, const float *d_w, float *d_out) {
    LFRV_API_BEGIN
    if (!ctx || !d_w || !d_out || mode < 0 || mode > 2) raise(LFRV_E_ARG, "bad argument");
    if ((mode != 1 && !d_x) || (mode != 0 && !d_dy)) raise(LFRV_E_ARG, "null operand");
    conv_single(ctx, mode, batch, H, W, Cin, Cout, ks, stride, d_x, d_dy, d_w, d_out);
    LFRV_API_END
}
