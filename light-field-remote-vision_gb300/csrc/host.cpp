// host.cpp -- C++ host orchestration of the lfrv solvers and the extern "C" boundary.
//
// The drivers follow the reference's control flow:
//   color_solve    : sr_synthesize_view (sources/super-resolution.cpp:54-338) and the cocolib stage
//                    functions it calls (sources/optimization.cu);
//   gradient_solve : IBR_gradient (sources/gradientIBR.cpp:12-150) with sources/gradientIBR.cu and
//                    possion_conj_grad (sources/solver.cu:526-699);
//   warp           : the GL warp exporter (sources/openGL/scene.cpp:1506-1586) restated as kernels.
// With cfg.faithful the reference's defects that change results are reproduced:
//   D5 the Sobel of compute_weights writes into the channel-0 dual variables (optimization.cu:1090-1092);
//   D6 the coverage accumulator is not cleared before the regulariser weight (optimization.cu:2262-2300);
//   D7 push-pull returns "filled - U" (optimization.cu:640-644);
//   D1 the CG loop of possion_conj_grad (beta == 1, alpha accumulator never cleared, 5 iterations).
// D2 (the FISTA extrapolation is overwritten by the next step, optimization.cu:1765-1767) never changes
// the result, so the extrapolation is not computed; the iterate simply advances.
#include "context.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

namespace lfrv {

void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) raise(e == cudaErrorMemoryAllocation ? LFRV_E_NOMEM : LFRV_E_CUDA, "%s: %s", what,
                                cudaGetErrorString(e));
}

std::atomic<unsigned long long> g_alloc_epoch{0};

void DevBuf::ensure(size_t b) {
    if (b <= bytes && p) return;
    release();
    if (b == 0) b = 16;
    LFRV_CUDA(cudaMalloc(&p, b));
    bytes = b;
    ++g_alloc_epoch;
}

void DevBuf::release() {
    if (p) {
        cudaFree(p);
        ++g_alloc_epoch;
    }
    p = nullptr;
    bytes = 0;
}

void KernelProfiler::init(int slots) {
    if (!ev.empty()) return;
    ev.resize(2 * (size_t)slots);
    for (auto &e : ev) LFRV_CUDA(cudaEventCreate(&e));
    recs.reserve(slots);
}

void KernelProfiler::destroy() {
    for (auto &e : ev) cudaEventDestroy(e);
    ev.clear();
    reset();
}

void KernelProfiler::reset() {
    recs.clear();
    next = 0;
    names.clear();
    ms.clear();
    count.clear();
}

void KernelProfiler::fold() {
    for (const auto &r : recs) {
        float t = 0.f;
        LFRV_CUDA(cudaEventSynchronize(ev[2 * r.slot + 1]));
        LFRV_CUDA(cudaEventElapsedTime(&t, ev[2 * r.slot], ev[2 * r.slot + 1]));
        size_t k = 0;
        while (k < names.size() && names[k] != r.name) ++k;
        if (k == names.size()) {
            names.push_back(r.name);
            ms.push_back(0.0);
            count.push_back(0);
        }
        ms[k] += t;
        count[k] += 1;
    }
    recs.clear();
    next = 0;
}

int KernelProfiler::begin(const char *name, cudaStream_t st) {
    if (2 * (size_t)(next + 1) > ev.size()) fold();
    const int slot = next++;
    cudaEventRecord(ev[2 * slot], st);
    recs.push_back({name, slot});
    return slot;
}

void KernelProfiler::end(int slot, cudaStream_t st) {
    if (slot >= 0) cudaEventRecord(ev[2 * slot + 1], st);
}

ProfScope::ProfScope(LaunchCounter &lc, const char *name, cudaStream_t s) : p(lc.prof), slot(-1), st(s) {
    if (p) slot = p->begin(name, st);
}

ProfScope::~ProfScope() {
    if (p) p->end(slot, st);
}

static void swap_buf(DevBuf &a, DevBuf &b) {
    std::swap(a.p, b.p);
    std::swap(a.bytes, b.bytes);
}

static GridBarrier fresh_barrier(lfrv_ctx *c);
static float *view_gradients(lfrv_ctx *c, const Geometry &G, const float *img, cudaStream_t st);
// Pinned host copy of a context's first 8 reduction sums (allocated on first use, freed with the context).
static double *host_sums(lfrv_ctx *c) {
    if (!c->host_sums) LFRV_CUDA(cudaMallocHost(reinterpret_cast<void **>(&c->host_sums), sizeof(double) * 8));
    return c->host_sums;
}

// The side stream: work of a call that depends only on its inputs runs there, between an event recorded on the
// context stream (fork) and one the context stream waits for (join). Created on first use.
static cudaStream_t side_stream(lfrv_ctx *c) {
    if (!c->side_stream) {
        LFRV_CUDA(cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking));
        LFRV_CUDA(cudaEventCreateWithFlags(&c->side_fork, cudaEventDisableTiming));
        LFRV_CUDA(cudaEventCreateWithFlags(&c->side_join, cudaEventDisableTiming));
    }
    return c->side_stream;
}

static void destroy_side_stream(lfrv_ctx *c) {
    if (!c->side_stream) return;
    cudaStreamSynchronize(c->side_stream);
    cudaStreamDestroy(c->side_stream);
    cudaEventDestroy(c->side_fork);
    cudaEventDestroy(c->side_join);
    c->side_stream = nullptr;
}

static void check_launch(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) raise(LFRV_E_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
}

static void sync(lfrv_ctx *c) { LFRV_CUDA(cudaStreamSynchronize(c->stream)); }

// Clears a caller's statistics, keeping its energy-trace request (buffer and capacity).
static void reset_stats(lfrv_stats *st) {
    if (!st) return;
    double *buf = st->energy_trace;
    const int cap = st->trace_capacity;
    std::memset(st, 0, sizeof(*st));
    st->energy_trace = buf;
    st->trace_capacity = cap;
}

// The caller's energy-trace request of this call: the device buffer (ws.trace) for its entries, or nullptr.
static double *trace_request(lfrv_ctx *c, lfrv_stats *st) {
    if (!st || !st->energy_trace || st->trace_capacity <= 0) return nullptr;
    c->ws.trace.ensure(sizeof(double) * (size_t)st->trace_capacity);
    c->pending.stats = st;
    c->pending.trace_host = st->energy_trace;
    c->pending.trace_cap = st->trace_capacity;
    c->pending.trace_len = -1;
    return c->ws.trace.as<double>();
}

// ------------------------------------------------------------------ geometry and validation
static Geometry geometry(const lfrv_config &cfg) {
    if (cfg.nchannels != 3) raise(LFRV_E_ARG, "nchannels must be 3 (sources/config.cpp:116), got %d", cfg.nchannels);
    if (cfg.w <= 0 || cfg.h <= 0) raise(LFRV_E_ARG, "bad view size %d x %d", cfg.w, cfg.h);
    if (cfg.dsf < 1 || cfg.dsf > 4) raise(LFRV_E_ARG, "dsf must be in 1..4, got %d", cfg.dsf);
    if (cfg.nviews < 1 || cfg.nviews > 255) raise(LFRV_E_ARG, "nviews must be in 1..255, got %d", cfg.nviews);
    if ((long long)cfg.w * cfg.h >= (1ll << 24)) raise(LFRV_E_ARG, "views larger than 2^24 pixels are not supported");
    Geometry G;
    G.V = cfg.nviews;
    G.w = cfg.w;
    G.h = cfg.h;
    G.n = cfg.w * cfg.h;
    G.dsf = cfg.dsf;
    G.W = cfg.w * cfg.dsf;
    G.H = cfg.h * cfg.dsf;
    G.N = (size_t)G.W * G.H;
    return G;
}

static void check_solver_options(const lfrv_config &cfg) {
    if (cfg.dw_type != 0) raise(LFRV_E_ARG, "dw_type %d: only 0 exists upstream (optimization.cu:1141-1147)", cfg.dw_type);
    if (cfg.niter < 0 || cfg.nmeta_iter < 0) raise(LFRV_E_ARG, "negative iteration count");
    if (!(cfg.lambda > 0.0f)) raise(LFRV_E_ARG, "lambda must be > 0");
    if (cfg.bf16_storage != 0 && cfg.bf16_storage != 1) raise(LFRV_E_ARG, "bf16_storage must be 0 or 1");
}

// ------------------------------------------------------------------ reductions
static double *partial_buf(lfrv_ctx *c, size_t count) {
    c->ws.partial.ensure(sizeof(double) * std::max<size_t>(count, 1));
    return c->ws.partial.as<double>();
}

// Reduces `count` partials at `partial` into sums[slot] on the device.
static void reduce_to(lfrv_ctx *c, int count, const double *partial, int slot) {
    c->ws.sums.ensure(sizeof(double) * 64);
    launch_reduce_final(count, partial, c->ws.sums.as<double>() + slot, c->stream, c->launches);
    check_launch("reduce");
}

static void read_sums(lfrv_ctx *c, double *host, int count) {
    LFRV_CUDA(cudaMemcpyAsync(host, c->ws.sums.p, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
}

// ------------------------------------------------------------------ inverse footprint map
static void geometry_key(const Geometry &G, long long key[5]) {
    key[0] = G.W;
    key[1] = G.H;
    key[2] = G.dsf;
    key[3] = G.V;
    key[4] = G.n;
}

// The inverse map's buffers for geometry G (allocated on first use).
static Buckets bucket_buffers(lfrv_ctx *c, const Geometry &G) {
    Workspace &ws = c->ws;
    const int ks = G.dsf + 1;
    Buckets B;
    B.BW = G.W + ks - 1;
    B.BH = G.H + ks - 1;
    B.nb = B.BW * B.BH;
    ws.b_count.ensure(sizeof(unsigned int) * B.nb);
    ws.b_start.ensure(sizeof(unsigned int) * (B.nb + 1));
    ws.b_entries.ensure(sizeof(unsigned int) * (size_t)G.V * G.n);
    const int nblk = (B.nb + 1023) / 1024;
    ws.b_aux.ensure(sizeof(unsigned int) * (4 * (size_t)nblk + 4 * 1024 + 16));
    unsigned int *aux = ws.b_aux.as<unsigned int>();
    B.count = ws.b_count.as<unsigned int>();
    B.start = ws.b_start.as<unsigned int>();
    B.entries = ws.b_entries.as<unsigned int>();
    B.mask_words = (G.V + 63) / 64;
    ws.b_mask.ensure(sizeof(unsigned long long) * B.nb * B.mask_words);
    B.mask = ws.b_mask.as<unsigned long long>();
    B.block_sums = aux;
    B.block_offsets = aux + nblk;
    B.block_sums2 = aux + 2 * nblk;
    B.block_offsets2 = aux + 2 * nblk + 1024;
    B.total = aux + 2 * nblk + 2048;
    B.total2 = aux + 2 * nblk + 2049;
    return B;
}

static Buckets build_buckets(lfrv_ctx *c, const Geometry &G, const float *tau2) {
    Buckets B = bucket_buffers(c, G);
    long long key[5];
    geometry_key(G, key);
    const bool counted = c->buckets_counted && c->counted_tau == tau2 &&
                         std::memcmp(key, c->counted_geometry, sizeof(key)) == 0;
    c->buckets_counted = false;
    launch_bucket_build(G, tau2, B, c->stream, c->launches, counted);
    check_launch("bucket build");
    return B;
}

// ------------------------------------------------------------------ shared pieces
static void gaussian_kernel_init() {
    // gsl_kernel_gauss_1xn(11, 2.0) (cocolib/cocolib/common/gsl_matrix_convolutions.cpp:42-63), uploaded as float
    double kd[11], s = 0;
    for (int x = -5; x <= 5; ++x) {
        kd[x + 5] = std::exp(-0.5 * x * x / 4.0);
        s += kd[x + 5];
    }
    float k[11];
    for (int i = 0; i < 11; ++i) k[i] = (float)(kd[i] / s);
    set_gaussian(k);
}

struct ColorBuffers {
    float *U, *Ua, *Ub, *P, *Pa, *F, *g, *g0, *tmp, *cov, *norm, *Xq, *gx, *gy, *res, *wgt, *Uprev, *Uprev_meta;
    uint8_t *vis;
};

static ColorBuffers color_buffers(lfrv_ctx *c, const Geometry &G) {
    Workspace &ws = c->ws;
    const size_t N = G.N, f = sizeof(float);
    ws.U.ensure(3 * N * f);
    ws.Ua.ensure(3 * N * f);
    ws.Ub.ensure(3 * N * f);
    ws.Uprev.ensure(6 * N * f);
    ws.P.ensure(6 * N * f);
    ws.Pa.ensure(6 * N * f);
    ws.F.ensure(3 * N * f);
    ws.g.ensure(N * f);
    ws.g0.ensure(N * f);
    ws.tmp.ensure(N * f);
    ws.cov.ensure(N * f);
    ws.norm.ensure(N * f);
    ws.Xq.ensure(2 * N * f);
    ws.gx.ensure(N * f);
    ws.gy.ensure(N * f);
    ws.vis.ensure(N);
    ws.wgt.ensure((size_t)G.V * G.n * f);
    ws.res.ensure((size_t)G.V * 3 * G.n * f);
    ColorBuffers b;
    b.U = ws.U.as<float>();
    b.Ua = ws.Ua.as<float>();
    b.Ub = ws.Ub.as<float>();
    b.P = ws.P.as<float>();
    b.Pa = ws.Pa.as<float>();
    b.F = ws.F.as<float>();
    b.g = ws.g.as<float>();
    b.g0 = ws.g0.as<float>();
    b.tmp = ws.tmp.as<float>();
    b.cov = ws.cov.as<float>();
    b.norm = ws.norm.as<float>();
    b.Xq = ws.Xq.as<float>();
    b.gx = ws.gx.as<float>();
    b.gy = ws.gy.as<float>();
    b.vis = ws.vis.as<uint8_t>();
    b.wgt = ws.wgt.as<float>();
    b.res = ws.res.as<float>();
    b.Uprev = ws.Uprev.as<float>();
    b.Uprev_meta = ws.Uprev.as<float>() + 3 * N;
    return b;
}

// Sobel of the luminance of U into (gx, gy) with visibility mask; optional sum of |gx| + |gy| into sums[slot].
static void sobel_target(lfrv_ctx *c, const Geometry &G, const float *U, float *gx, float *gy, const uint8_t *vis,
                         int abs_slot) {
    double *part = nullptr;
    const int np = sobel_partials(G.W, G.H);
    if (abs_slot >= 0) part = partial_buf(c, np);
    launch_sobel(G.W, G.H, 1, U, 0, G.N, gx, gy, 0, vis, part, c->stream, c->launches);
    check_launch("sobel");
    if (abs_slot >= 0) reduce_to(c, np, part, abs_slot);
}

// Weighted residuals of every view at U (and the intensity energy into sums[slot]).
static void residual(lfrv_ctx *c, const Geometry &G, const float *U, const float *img, const float *tau2,
                     const float *wgt, float s2, float *res, int slot, bool splat_set = false) {
    const int np = residual_partials(G);
    double *part = partial_buf(c, np);
    launch_residual(G, U, img, tau2, wgt, s2, res, part, c->stream, c->launches, splat_set);
    check_launch("residual");
    reduce_to(c, np, part, slot);
}

// ------------------------------------------------------------------ autotuner
// Picks the persistent-ROF instantiation (iterations per super-step, block size) for a W x H image: each candidate
// runs 16 iterations on a scratch copy of the state (U, P, F, g), timed with CUDA events on the context stream;
// the fastest is cached per image size in the context. The solver's own buffers are not touched.
static int rof_autotune(lfrv_ctx *c, int W, int H, float tau, float sigma, float lam, const float *U, const float *P,
                        const float *F, const float *g) {
    const long long key = ((long long)W << 32) | (unsigned)H;
    auto it = c->rof_tuned.find(key);
    if (it != c->rof_tuned.end()) return it->second;
    const size_t N = (size_t)W * H;
    c->ws.tune.ensure(sizeof(float) * 18 * N);
    float *U0 = c->ws.tune.as<float>(), *U1 = U0 + 3 * N, *P0 = U1 + 3 * N, *P1 = P0 + 6 * N;
    cudaStream_t s = c->stream;
    cudaEvent_t e0, e1;
    LFRV_CUDA(cudaEventCreate(&e0));
    LFRV_CUDA(cudaEventCreate(&e1));
    int best = rof_default_variant();
    float best_ms = 1e30f;
    LaunchCounter quiet;  // trial launches are not the caller's kernels
    for (int v = 0; v < rof_variant_count(); ++v) {
        LFRV_CUDA(cudaMemcpyAsync(U0, U, sizeof(float) * 3 * N, cudaMemcpyDeviceToDevice, s));
        LFRV_CUDA(cudaMemcpyAsync(P0, P, sizeof(float) * 6 * N, cudaMemcpyDeviceToDevice, s));
        const GridBarrier gb = fresh_barrier(c);
        LFRV_CUDA(cudaEventRecord(e0, s));
        const cudaError_t e = launch_rof_persistent(W, H, 16, tau, sigma, lam, U0, P0, U1, P1, F, g, gb, v, s, quiet);
        LFRV_CUDA(cudaEventRecord(e1, s));
        if (e != cudaSuccess) {
            cudaGetLastError();
            continue;  // a variant that cannot launch here (occupancy) is skipped
        }
        LFRV_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        LFRV_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->rof_tuned[key] = best;
    return best;
}

// The FGP's counterpart of rof_autotune: every instantiation of the arithmetic in use, timed on scratch copies of
// the dual (16 iterations) on first use per image size; the fastest is cached. All give the same iterates.
static int fgp_autotune(lfrv_ctx *c, int W, int H, bool extended, const float *F, const float *lam, const float *linv,
                        const float *g, const double *P) {
    const long long key = ((long long)W << 33) | ((long long)H << 1) | (extended ? 1 : 0);
    auto it = c->fgp_tuned.find(key);
    if (it != c->fgp_tuned.end()) return it->second;
    const size_t N = (size_t)W * H;
    c->ws.tune.ensure(sizeof(double) * 24 * N + sizeof(float) * 3 * N);
    double *P0 = c->ws.tune.as<double>(), *P1 = P0 + 6 * N, *Q0 = P1 + 6 * N, *Q1 = Q0 + 6 * N;
    float *U = reinterpret_cast<float *>(Q1 + 6 * N);
    cudaStream_t s = c->stream;
    cudaEvent_t e0, e1;
    LFRV_CUDA(cudaEventCreate(&e0));
    LFRV_CUDA(cudaEventCreate(&e1));
    int best = tv_fgp_default_variant(extended);
    float best_ms = 1e30f;
    LaunchCounter quiet;  // trial launches are not the caller's kernels
    for (int v = 0; v < tv_fgp_variant_count(extended); ++v) {
        LFRV_CUDA(cudaMemcpyAsync(P0, P, sizeof(double) * 6 * N, cudaMemcpyDeviceToDevice, s));
        const GridBarrier gb = fresh_barrier(c);
        LFRV_CUDA(cudaEventRecord(e0, s));
        const cudaError_t e = launch_tv_fgp(W, H, 16, F, lam, linv, g, P0, P1, Q0, Q1, U, gb, s, quiet, extended, v);
        LFRV_CUDA(cudaEventRecord(e1, s));
        if (e != cudaSuccess) {
            cudaGetLastError();
            continue;  // a variant that cannot launch here (occupancy) is skipped
        }
        LFRV_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        LFRV_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->fgp_tuned[key] = best;
    return best;
}

// ------------------------------------------------------------------ gradient data term (dt_beta)
// Buffers of the gradient data term (vtv_sr_dataterm_gradients, sources/optimization.cu:1969-2116) and of the
// gradient term of the energy (:1610-1700); empty when dt_beta == 0.
struct GradientTermBuffers {
    bool on = false;
    const float *vgrad = nullptr;  // Sobel of each view's luminance, 2 x n per view
    float *lapU = nullptr, *resg = nullptr, *ugrad = nullptr;
};

static GradientTermBuffers gradient_term_buffers(lfrv_ctx *c, const lfrv_config &cfg, const Geometry &G,
                                                 const float *img) {
    GradientTermBuffers t;
    if (cfg.dt_beta == 0.0f) return t;
    Workspace &ws = c->ws;
    ws.lapU.ensure(sizeof(float) * 3 * G.N);
    ws.resg.ensure(sizeof(float) * 3 * (size_t)G.V * G.n);
    ws.ugrad.ensure(sizeof(float) * 2 * G.N);
    t.on = true;
    t.vgrad = view_gradients(c, G, img, c->stream);
    t.lapU = ws.lapU.as<float>();
    t.resg = ws.resg.as<float>();
    t.ugrad = ws.ugrad.as<float>();
    return t;
}

// Residuals of the gradient data term for the current U; the term is applied by the data-term kernel.
static GradTerm gradient_residuals(lfrv_ctx *c, const lfrv_config &cfg, const Geometry &G,
                                   const GradientTermBuffers &t, const float *U, const float *img, const float *tau2,
                                   const float *wgt) {
    GradTerm gt{nullptr, 0.f, 0.f, 0};
    if (!(cfg.dt_beta > 0.0f)) return gt;  // the ISTA step runs the term for dt_beta > 0 (optimization.cu:1781)
    launch_laplacian(G.W, G.H, 3, U, t.lapU, c->stream, c->launches);
    launch_residual_grad(G, t.lapU, img, tau2, wgt, cfg.gw_type != 0, t.resg, c->stream, c->launches);
    check_launch("gradient residual");
    gt.resg = t.resg;
    gt.beta = cfg.dt_beta;
    gt.step = cfg.gradient_step;
    gt.gw = cfg.gw_type != 0;
    return gt;
}

// Gradient term of the reference energy into sums[slot]: Sobel of the luminance of U (no mask) gathered per view
// and compared with the views' Sobel.
static void energy_gradients(lfrv_ctx *c, const lfrv_config &cfg, const Geometry &G, const GradientTermBuffers &t,
                             const float *U, const float *tau2, const float *wgt, int slot) {
    launch_sobel(G.W, G.H, 1, U, 0, G.N, t.ugrad, t.ugrad + G.N, 0, nullptr, nullptr, c->stream, c->launches);
    const int np = energy_grad_partials(G);
    double *part = partial_buf(c, np);
    launch_energy_grad(G, t.ugrad, t.vgrad, tau2, wgt, cfg.sigma_sensor * cfg.sigma_sensor, cfg.gw_type != 0, part,
                       c->stream, c->launches);
    check_launch("energy gradient term");
    reduce_to(c, np, part, slot);
}

// ------------------------------------------------------------------ IBR_color, corrected mode
// The corrected IBR_color solve of one target (kernels_tv.cu), held in the workspace of context c and driven one
// outer iteration at a time, so that several targets on their own contexts can advance in lockstep with one host
// synchronisation per round: eval() enqueues the energy and certificate of the current iterate and their copy to
// host memory; after the stream has completed, decide() reads them, records the trace and the stop decision; step()
// enqueues one FISTA step (its FGP dual solve in one persistent launch).
struct TvSolve {
    lfrv_ctx *c = nullptr;
    lfrv_config cfg{};
    Geometry G{};
    const float *img = nullptr, *tau2 = nullptr;
    Buckets B{};
    ColorBuffers b{};
    float *u = nullptr, *up = nullptr, *gf = nullptr, *gfp = nullptr, *D = nullptr, *lam = nullptr, *linv = nullptr;
    double *P0 = nullptr, *P1 = nullptr, *Q0 = nullptr, *Q1 = nullptr;
    double t = 1.0, E_prev = 1e300, E = 0.0, gap = 1e300;
    bool extended = false, done = false;
    int k = 0, npart = 0;
    lfrv_stats *st = nullptr;  // energy trace destination (optional)
    int trace_pos = 0;

    // set-up for one meta iteration on ws.U (weights and regulariser weight computed): the metric, u = clamp(U),
    // the FISTA history and, for the first meta iteration, a zero dual
    void begin(int meta) {
        Workspace &ws = c->ws;
        const size_t N = G.N, N3 = 3 * N;
        cudaStream_t s = c->stream;
        // 15 N floats (u, u_prev, grad f, grad f_prev, D, lam, 1/L), then 24 N doubles (p, its ping-pong copy, q x 2)
        const size_t fbytes = (sizeof(float) * 15 * N + 255) / 256 * 256;
        ws.tv.ensure(fbytes + sizeof(double) * 24 * N);
        u = ws.tv.as<float>();
        up = u + N3;
        gf = up + N3;
        gfp = gf + N3;
        D = gfp + N3;
        lam = D + N;
        linv = lam + N;
        P0 = reinterpret_cast<double *>(ws.tv.as<char>() + fbytes);
        P1 = P0 + 6 * N;
        Q0 = P1 + 6 * N;
        Q1 = Q0 + 6 * N;
        launch_tv_metric(G, B, tau2, b.wgt, as2(), cfg.lambda, D, lam, linv, s, c->launches);
        check_launch("tv metric");
        launch_tv_clamp(N3, ws.U.as<float>(), u, s, c->launches);
        // u_prev = u and grad f(u_prev) = 0: the first step (theta = 0) reads them only through zero factors
        LFRV_CUDA(cudaMemcpyAsync(up, u, sizeof(float) * N3, cudaMemcpyDeviceToDevice, s));
        LFRV_CUDA(cudaMemsetAsync(gfp, 0, sizeof(float) * N3, s));
        if (meta == 0) LFRV_CUDA(cudaMemsetAsync(P0, 0, sizeof(double) * 6 * N, s));
        npart = tv_gap_partials(G.W, G.H);
        t = 1.0;
        E_prev = 1e300;
        extended = false;
        done = false;
        k = 0;
    }
    float as2() const { return cfg.dt_alpha * cfg.sigma_sensor * cfg.sigma_sensor; }
    void eval() {
        const float s2 = cfg.sigma_sensor * cfg.sigma_sensor;
        residual(c, G, u, img, tau2, b.wgt, s2, b.res, 1, true);
        launch_tv_gradf(G, B, tau2, b.res, as2(), gf, c->stream, c->launches);
        check_launch("tv data gradient");
        double *part = partial_buf(c, 3 * (size_t)npart);
        launch_tv_gap(G.W, G.H, u, gf, P0, b.g, cfg.lambda, part, c->stream, c->launches);
        check_launch("tv gap");
        for (int q = 0; q < 3; ++q) reduce_to(c, npart, part + (size_t)q * npart, 4 + q);
        LFRV_CUDA(cudaMemcpyAsync(host_sums(c), c->ws.sums.p, sizeof(double) * 7, cudaMemcpyDeviceToHost, c->stream));
    }
    // after the stream has completed: true when the solve has stopped (gap reached or the cap)
    bool decide() {
        const double *sums = host_sums(c);
        const double f = 0.5 * (double)cfg.dt_alpha * sums[1];
        E = f + (double)cfg.lambda * sums[4];
        const double gap_abs = (double)cfg.lambda * (sums[4] - sums[5]) + sums[6];
        gap = E > 0 ? gap_abs / E : 1e300;
        if (st && st->energy_trace && trace_pos < st->trace_capacity) st->energy_trace[trace_pos++] = E;
        if (!std::isfinite(E) || !std::isfinite(gap))
            raise(LFRV_E_NONFINITE, "non-finite energy in the corrected IBR_color solve");
        done = k >= cfg.niter || (cfg.cg_gap_tol > 0 && gap <= cfg.cg_gap_tol);
        return done;
    }
    void step() {
        cudaStream_t s = c->stream;
        if (E > E_prev) t = 1.0;  // function-value restart of the momentum
        E_prev = E;
        const double t1 = 0.5 * (1.0 + std::sqrt(1.0 + 4.0 * t * t));
        const float theta = (float)((t - 1.0) / t1);
        t = t1;
        launch_tv_fstep(G.W, G.H, u, up, gf, gfp, D, theta, b.F, s, c->launches);
        check_launch("tv step");
        std::swap(u, up);
        std::swap(gf, gfp);
        // FP32 dual arithmetic while the gap is far above FP32's floor, double-float once it nears it (the switch
        // only changes rounding, not the iteration)
        extended = extended || gap < kTvExtendedBelow;
        const int variant = fgp_autotune(c, G.W, G.H, extended, b.F, lam, linv, b.g, P0);
        const GridBarrier gb = fresh_barrier(c);  // after the autotuner's trial launches, which use the barrier too
        LFRV_CUDA(launch_tv_fgp(G.W, G.H, kTvInnerIterations, b.F, lam, linv, b.g, P0, P1, Q0, Q1, u, gb, s,
                                c->launches, extended, variant));
        ++k;
    }
    // the solution back into ws.U
    void finish() {
        LFRV_CUDA(cudaMemcpyAsync(c->ws.U.p, u, sizeof(float) * 3 * G.N, cudaMemcpyDeviceToDevice, c->stream));
    }

    // The whole loop (begun) as one CUDA graph with the stop test on the device: eval and k_tv_decide, then a
    // conditional WHILE node whose body is the FISTA step (theta from the device state; u and grad f kept as the
    // previous ones by copies, so the body's buffers never change), a conditional IF node choosing the FGP's
    // arithmetic (double-float or FP32, each autotuned beforehand), eval and k_tv_decide again. No host round trip
    // per step; the same arithmetic and decisions as eval / decide / step. False when the graph cannot be built
    // here (the caller then runs the host loop); the solve's state is unchanged then.
    bool run_graph() {
        if (c->launches.prof) return false;  // per-kernel profiling brackets launches with events
        cudaStream_t s = c->stream;
        Workspace &ws = c->ws;
        const size_t N = G.N, N3 = 3 * N;
        // everything the captured launches use, allocated and tuned before the capture
        const int vf = fgp_autotune(c, G.W, G.H, false, b.F, lam, linv, b.g, P0);
        const int vd = fgp_autotune(c, G.W, G.H, true, b.F, lam, linv, b.g, P0);
        partial_buf(c, std::max<size_t>((size_t)residual_partials(G), 3 * (size_t)npart));
        ws.sums.ensure(sizeof(double) * 64);
        ws.tvloop.ensure(sizeof(TvLoopState));
        const int cap = (st && st->energy_trace) ? st->trace_capacity : 0;
        if (cap > 0) ws.trace.ensure(sizeof(double) * cap);
        TvLoopState *loop = ws.tvloop.as<TvLoopState>();
        TvLoopState init{};
        init.t = t;
        init.E_prev = E_prev;
        init.E = E;
        init.gap = gap;
        init.k = k;
        init.extended = extended ? 1 : 0;
        init.trace_pos = trace_pos;
        LFRV_CUDA(cudaMemcpyAsync(loop, &init, sizeof(init), cudaMemcpyHostToDevice, s));
        LFRV_CUDA(cudaStreamSynchronize(s));
        double *dtrace = cap > 0 ? ws.trace.as<double>() : nullptr;
        const long long n0 = c->launches.n;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<cudaGraph_t> pieces;
        bool ok = false;
        long long n_pro = 0, n_body = 0;
        do {
            if (cudaGraphCreate(&g, 0) != cudaSuccess) break;
            cudaGraphConditionalHandle h_loop, h_ext;
            if (cudaGraphConditionalHandleCreate(&h_loop, g, 0, 0) != cudaSuccess ||
                cudaGraphConditionalHandleCreate(&h_ext, g, 0, 0) != cudaSuccess)
                break;
            auto capture = [&](auto &&fn, long long &count) -> cudaGraph_t {
                cudaGraph_t piece = nullptr;
                const long long before = c->launches.n;
                if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return nullptr;
                fn();
                if (cudaStreamEndCapture(s, &piece) != cudaSuccess) return nullptr;
                count += c->launches.n - before;
                pieces.push_back(piece);
                return piece;
            };
            auto eval_decide = [&]() {
                const float s2 = cfg.sigma_sensor * cfg.sigma_sensor;
                residual(c, G, u, img, tau2, b.wgt, s2, b.res, 1, true);
                launch_tv_gradf(G, B, tau2, b.res, as2(), gf, s, c->launches);
                double *part = partial_buf(c, 3 * (size_t)npart);
                launch_tv_gap(G.W, G.H, u, gf, P0, b.g, cfg.lambda, part, s, c->launches);
                for (int q = 0; q < 3; ++q) reduce_to(c, npart, part + (size_t)q * npart, 4 + q);
                launch_tv_decide(ws.sums.as<double>(), (double)cfg.dt_alpha, (double)cfg.lambda, cfg.cg_gap_tol,
                                 cfg.niter, loop, dtrace, cap, h_loop, h_ext, s, c->launches);
            };
            auto fgp = [&](bool ext, int variant) {
                const GridBarrier gb = fresh_barrier(c);
                cudaError_t e = launch_tv_fgp(G.W, G.H, kTvInnerIterations, b.F, lam, linv, b.g, P0, P1, Q0, Q1, u, gb,
                                              s, c->launches, ext, variant);
                if (e != cudaSuccess) cudaGetLastError();
            };
            long long n_fgp = 0;
            cudaGraph_t g_pro = capture(eval_decide, n_pro);
            cudaGraph_t g_step = capture(
                [&]() {
                    launch_tv_fstep(G.W, G.H, u, up, gf, gfp, D, 0.f, b.F, s, c->launches, loop);
                    cudaMemcpyAsync(up, u, sizeof(float) * N3, cudaMemcpyDeviceToDevice, s);
                    cudaMemcpyAsync(gfp, gf, sizeof(float) * N3, cudaMemcpyDeviceToDevice, s);
                },
                n_body);
            long long n_dummy = 0;
            cudaGraph_t g_df = capture([&]() { fgp(true, vd); }, n_fgp);
            cudaGraph_t g_f = capture([&]() { fgp(false, vf); }, n_dummy);
            cudaGraph_t g_ev = capture(eval_decide, n_body);
            if (!g_pro || !g_step || !g_df || !g_f || !g_ev) break;
            n_body += n_fgp;
            cudaGraphNode_t n_p, n_w;
            if (cudaGraphAddChildGraphNode(&n_p, g, nullptr, 0, g_pro) != cudaSuccess) break;
            cudaGraphNodeParams wp = {};
            wp.type = cudaGraphNodeTypeConditional;
            wp.conditional.handle = h_loop;
            wp.conditional.type = cudaGraphCondTypeWhile;
            wp.conditional.size = 1;
            if (cudaGraphAddNode(&n_w, g, &n_p, nullptr, 1, &wp) != cudaSuccess) break;
            cudaGraph_t body = wp.conditional.phGraph_out[0];
            cudaGraphNode_t b_step, b_if, b_ev;
            if (cudaGraphAddChildGraphNode(&b_step, body, nullptr, 0, g_step) != cudaSuccess) break;
            cudaGraphNodeParams ip = {};
            ip.type = cudaGraphNodeTypeConditional;
            ip.conditional.handle = h_ext;
            ip.conditional.type = cudaGraphCondTypeIf;
            ip.conditional.size = 2;
            if (cudaGraphAddNode(&b_if, body, &b_step, nullptr, 1, &ip) != cudaSuccess) break;
            cudaGraphNode_t b_df, b_f;
            if (cudaGraphAddChildGraphNode(&b_df, ip.conditional.phGraph_out[0], nullptr, 0, g_df) != cudaSuccess ||
                cudaGraphAddChildGraphNode(&b_f, ip.conditional.phGraph_out[1], nullptr, 0, g_f) != cudaSuccess)
                break;
            if (cudaGraphAddChildGraphNode(&b_ev, body, &b_if, 1, g_ev) != cudaSuccess) break;
            if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) break;
            ok = true;
        } while (false);
        for (cudaGraph_t piece : pieces) cudaGraphDestroy(piece);
        if (!ok) {
            cudaGetLastError();
            if (exec) cudaGraphExecDestroy(exec);
            if (g) cudaGraphDestroy(g);
            c->launches.n = n0;
            return false;
        }
        LFRV_CUDA(cudaGraphLaunch(exec, s));
        TvLoopState fin{};
        LFRV_CUDA(cudaMemcpyAsync(&fin, loop, sizeof(fin), cudaMemcpyDeviceToHost, s));
        LFRV_CUDA(cudaStreamSynchronize(s));
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(g);
        // launches: the prologue once, the body once per step taken
        c->launches.n = n0 + n_pro + (long long)(fin.k - k) * n_body;
        if (fin.err) raise(LFRV_E_NONFINITE, "non-finite energy in the corrected IBR_color solve");
        if (cap > 0 && fin.trace_pos > trace_pos)
            LFRV_CUDA(cudaMemcpy(st->energy_trace + trace_pos, dtrace + trace_pos,
                                 sizeof(double) * (fin.trace_pos - trace_pos), cudaMemcpyDeviceToHost));
        t = fin.t;
        E_prev = fin.E_prev;
        E = fin.E;
        gap = fin.gap;
        k = fin.k;
        extended = fin.extended != 0;
        trace_pos = fin.trace_pos;
        done = true;
        return true;
    }
};

// ------------------------------------------------------------------ IBR_color
// defer (corrected mode with one meta iteration): the set-up runs, then *defer receives the solve, begun, and the
// caller drives it and copies the result (TvSolve::finish puts it into the context's ws.U).
static void color_solve(lfrv_ctx *c, const lfrv_config &cfg, const float *img, const float *tau2, const float *dp2,
                        const float *init, float *out, lfrv_stats *st, TvSolve *defer = nullptr) {
    check_solver_options(cfg);
    if (cfg.bf16_storage) raise(LFRV_E_ARG, "bf16_storage applies to IBR_gradient only");
    if (!cfg.faithful && cfg.dt_beta != 0.0f)
        raise(LFRV_E_ARG, "corrected IBR_color solves the intensity objective: dt_beta must be 0");
    const Geometry G = geometry(cfg);
    const size_t N = G.N;
    cudaStream_t s = c->stream;
    Workspace &ws = c->ws;
    const bool faithful = cfg.faithful != 0;
    const float sigma = cfg.sigma_sensor, s2 = cfg.sigma_sensor * cfg.sigma_sensor;
    const Buckets B = build_buckets(c, G, tau2);
    ColorBuffers b = color_buffers(c, G);
    const GradientTermBuffers gtb = gradient_term_buffers(c, cfg, G, img);
    LFRV_CUDA(cudaMemsetAsync(b.U, 0, 3 * N * sizeof(float), s));
    LFRV_CUDA(cudaMemsetAsync(b.P, 0, 6 * N * sizeof(float), s));
    LFRV_CUDA(cudaMemsetAsync(b.Xq, 0, 2 * N * sizeof(float), s));
    LFRV_CUDA(cudaMemsetAsync(b.vis, 0, N, s));
    LFRV_CUDA(cudaMemsetAsync(b.gx, 0, N * sizeof(float), s));
    LFRV_CUDA(cudaMemsetAsync(b.gy, 0, N * sizeof(float), s));
    // gradient buffers of compute_weights: the channel-0 duals when faithful (D5)
    auto grad_x = [&]() { return faithful ? ws.P.as<float>() : b.gx; };
    auto grad_y = [&]() { return faithful ? ws.P.as<float>() + N : b.gy; };
    auto compute_weights = [&]() {
        sobel_target(c, G, ws.U.as<float>(), grad_x(), grad_y(), b.vis, -1);
        launch_weights(G, grad_x(), grad_y(), tau2, dp2, sigma, cfg.ugrad_threshold, b.wgt, s, c->launches);
        check_launch("weights");
    };
    compute_weights();  // super-resolution.cpp:157, U = 0 and an empty visibility mask
    launch_coverage(G, B, tau2, b.cov, b.vis, s, c->launches);  // :160
    check_launch("coverage");
    // content of the reference's coverage accumulator (norm_mask) before the regulariser weight
    const float *norm_prior = b.cov;
    if (init) {
        LFRV_CUDA(cudaMemcpyAsync(ws.U.p, init, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    } else {
        launch_initial_image(G, B, tau2, img, b.wgt, ws.U.as<float>(), b.norm, s, c->launches);  // :165
        check_launch("initial image");
        norm_prior = b.norm;
        ws.pp_img.ensure(sizeof(float) * 3 * (N / 2 + 16));
        ws.pp_vis.ensure(N / 2 + 16 + N);
        ws.pp_tmp.ensure(sizeof(float) * 3 * (N / 2 + (size_t)G.W + 16));
        ws.pp_orig.ensure(sizeof(float) * 3 * N);
        PushPull pp;
        float *pi = ws.pp_img.as<float>();
        uint8_t *pv = ws.pp_vis.as<uint8_t>();
        pp.vis[0] = pv;
        pv += N;
        for (int l = 1; l <= 10; ++l) {
            const size_t sz = (size_t)(G.W >> l) * (G.H >> l);
            pp.img[l] = pi;
            pp.vis[l] = pv;
            pi += 3 * sz;
            pv += sz;
        }
        pp.tmp = ws.pp_tmp.as<float>();
        pp.orig = ws.pp_orig.as<float>();
        launch_push_pull(G.W, G.H, faithful, b.vis, ws.U.as<float>(), pp, s, c->launches);
        check_launch("push-pull");
    }
    if (!faithful) norm_prior = nullptr;
    if (cfg.early_exit) {
        LFRV_CUDA(cudaMemcpyAsync(b.Uprev, ws.U.p, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
        LFRV_CUDA(cudaMemcpyAsync(b.Uprev_meta, ws.U.p, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    // primal-dual constants of coco_vtv_sr_iteration_fista_unstructured (optimization.cu:1739-1741)
    const float tau_pd = (float)(0.3 / std::sqrt(8.0)), sigma_pd = (float)(0.3 / std::sqrt(8.0));
    const float L = (float)(1.0 / cfg.lambda);
    const float lam_prox = (float)(1.0 / L);
    const float fscale = (float)(-1.0 / (double)(cfg.lambda * L));
    const float EPS = 1e-4f, MAX_DIFF = 1e-3f, PERCENT_MOVING = 0.01f;
    const int mp = moving_partials(N);

    // energy trace: one entry per FISTA iteration, written on the device (no host read per iteration)
    double *trace = trace_request(c, st);
    const int trace_cap = trace ? st->trace_capacity : 0;
    auto energy = [&](bool need_tv, int trace_slot = -1) -> float {
        // residual pass (also the data term input of the next iteration) + TV term of the reference energy
        residual(c, G, ws.U.as<float>(), img, tau2, b.wgt, s2, b.res, 1);
        const bool want_trace = trace_slot >= 0 && trace_slot < trace_cap;
        if (!need_tv && !want_trace) return 0.0f;
        sobel_target(c, G, ws.U.as<float>(), b.Xq, b.Xq + N, b.vis, 0);
        if (gtb.on) energy_gradients(c, cfg, G, gtb, ws.U.as<float>(), tau2, b.wgt, 3);
        if (want_trace) {
            launch_trace_energy(ws.sums.as<double>(), cfg.lambda, cfg.dt_alpha, cfg.dt_beta, gtb.on,
                                trace + trace_slot, s, c->launches);
            check_launch("trace energy");
        }
        if (!need_tv) return 0.0f;
        double sums[4] = {0, 0, 0, 0};
        read_sums(c, sums, gtb.on ? 4 : 2);
        const float e_tv = (float)sums[0], e_int = (float)sums[1], e_grad = (float)sums[3];
        return cfg.lambda * e_tv + cfg.dt_alpha * e_int + (gtb.on ? cfg.dt_beta * e_grad : 0.0f);
    };
    auto moving = [&](const float *a, const float *bb) -> int {
        double *part = partial_buf(c, mp);
        launch_moving(N, a, bb, MAX_DIFF, part, s, c->launches);
        check_launch("moving");
        reduce_to(c, mp, part, 2);
        double v[3];
        read_sums(c, v, 3);
        return (int)v[2];
    };

    // corrected mode: the true TV_F objective to a certified primal-dual gap (kernels_tv.cu); one call per meta
    // iteration on ws.U, returning the outer iterations run. Trace entries (the energy of every iterate, the start
    // included) are written to the caller's buffer from the host, where the energy is read for the stop test.
    double tv_gap_last = 0.0, tv_E = 0.0;
    int tv_trace_pos = 0;
    auto tv_solver = [&]() {
        TvSolve ts;
        ts.c = c;
        ts.cfg = cfg;
        ts.G = G;
        ts.img = img;
        ts.tau2 = tau2;
        ts.B = B;
        ts.b = b;
        ts.st = trace ? st : nullptr;
        ts.trace_pos = tv_trace_pos;
        return ts;
    };
    auto tv_meta = [&](int meta) -> int {
        TvSolve ts = tv_solver();
        ts.begin(meta);
        if (!ts.run_graph()) {
            for (;;) {
                ts.eval();
                sync(c);
                if (ts.decide()) break;
                ts.step();
            }
        }
        ts.finish();
        tv_E = ts.E;
        tv_gap_last = ts.gap;
        tv_trace_pos = ts.trace_pos;
        return ts.k;
    };
    float E = 0.0f, E_prev = 0.0f, E_prev_reweight = 0.0f;
    int total_k = 0, reason = 0, r = 0;
    const bool track = cfg.early_exit != 0;
    for (r = 0; r < cfg.nmeta_iter; ++r) {
        compute_weights();
        launch_regweight(G, B, tau2, b.wgt, norm_prior, s2, cfg.lambda_max_factor * cfg.lambda, cfg.lambda,
                         (float)G.V, b.g0, b.norm, s, c->launches);
        check_launch("regularizer weight");
        launch_blur(G.W, G.H, b.g0, b.tmp, b.g, s, c->launches);
        check_launch("blur");
        if (!faithful && defer) {
            *defer = tv_solver();
            defer->begin(0);
            return;
        }
        if (!faithful) {
            total_k += tv_meta(r);
            E = (float)tv_E;
            reason = (cfg.cg_gap_tol > 0 && tv_gap_last <= cfg.cg_gap_tol) ? 4 : 0;
            continue;
        }
        E = energy(true);
        E_prev = E;
        int k;
        for (k = 0; k < cfg.niter; ++k) {
            const GradTerm gt = gradient_residuals(c, cfg, G, gtb, ws.U.as<float>(), img, tau2, b.wgt);
            launch_dataterm_F(G, B, tau2, b.res, s2, cfg.dt_alpha, fscale, ws.U.as<float>(), b.F, nullptr, gt, s,
                              c->launches);
            check_launch("data term");
            // niter inner ROF iterations from Uq = U in one persistent launch over (Ua, P) <-> (Ub, Pa);
            // U itself stays the previous iterate (the moving-pixel test compares against it)
            LFRV_CUDA(cudaMemcpyAsync(ws.Ua.p, ws.U.p, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
            const int rv = rof_autotune(c, G.W, G.H, tau_pd, sigma_pd, lam_prox, ws.Ua.as<float>(), ws.P.as<float>(),
                                        b.F, b.g);
            const GridBarrier gb = fresh_barrier(c);
            LFRV_CUDA(launch_rof_persistent(G.W, G.H, cfg.niter, tau_pd, sigma_pd, lam_prox, ws.Ua.as<float>(),
                                            ws.P.as<float>(), ws.Ub.as<float>(), ws.Pa.as<float>(), b.F, b.g, gb, rv, s,
                                            c->launches));
            const bool odd = (rof_persistent_steps(cfg.niter, rv) & 1) != 0;
            const float *Ucur = odd ? ws.Ub.as<float>() : ws.Ua.as<float>();
            if (odd) swap_buf(ws.P, ws.Pa);
            int nM = 0;
            if (track) nM = moving(Ucur, ws.U.as<float>());
            // U <- the ROF result
            if (Ucur == ws.Ua.as<float>()) swap_buf(ws.U, ws.Ua);
            else if (Ucur == ws.Ub.as<float>()) swap_buf(ws.U, ws.Ub);
            ++total_k;
            E = energy(track, total_k - 1);
            if (!track) continue;
            if (E < EPS) {
                reason = 1;
                break;
            }
            const double rel = std::fabs((double)((E - E_prev) / E));
            if (rel < (double)EPS) {
                reason = 2;
                break;
            }
            E_prev = E;
            // sr_compare_images against R_prev (the iterate kept at the last non-breaking iteration)
            nM = moving(ws.U.as<float>(), b.Uprev);
            if ((float)nM / (float)N < PERCENT_MOVING) {
                reason = 3;
                break;
            }
            LFRV_CUDA(cudaMemcpyAsync(b.Uprev, ws.U.p, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
        }
        if (faithful) norm_prior = (k > 0) ? b.cov : b.norm;  // data term clears and re-accumulates the coverage
        if (!track) {
            if (r == cfg.nmeta_iter - 1) E = energy(true);  // reported energy of the final iterate
            continue;
        }
        if (E < EPS) {
            if (E_prev_reweight < EPS) break;
            E_prev_reweight = E;
            continue;
        }
        const int nM = moving(ws.U.as<float>(), b.Uprev_meta);
        if ((float)nM / (float)N < PERCENT_MOVING) break;
        LFRV_CUDA(cudaMemcpyAsync(b.Uprev_meta, ws.U.p, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    LFRV_CUDA(cudaMemcpyAsync(out, ws.U.p, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (trace && faithful) c->pending.trace_len = std::min(total_k, trace_cap);
    if (trace && !faithful) {  // the corrected solve wrote its trace from the host
        c->pending.trace_host = nullptr;
        st->trace_length = tv_trace_pos;
    }
    if (st) {
        st->outer_iterations = total_k;
        st->meta_iterations = std::min(r + 1, cfg.nmeta_iter);
        st->stop_reason = reason;
        st->energy = faithful ? (double)E : tv_E;
        st->gap = faithful ? 0.0 : tv_gap_last;
    }
}

// ------------------------------------------------------------------ IBR_gradient
// Device state of the persistent solvers, read back after the stream completes (lfrv::finish_stats):
// [0..2] CG delta, [3] CG energy, [4] CG certified gap, [5] CG iterations, [8] hole-fill iterations.
static double *solver_state(lfrv_ctx *c) {
    c->ws.state.ensure(sizeof(double) * 16);
    return c->ws.state.as<double>();
}

static GridBarrier fresh_barrier(lfrv_ctx *c) {
    // the arrival counter restarts for every launch; the error word is cleared only by the first launch
    // since the last check, so a timeout of an earlier launch of the same call is still reported
    c->ws.barrier.ensure(64);
    LFRV_CUDA(cudaMemsetAsync(c->ws.barrier.p, 0, c->pending.barrier ? 16 : 64, c->stream));
    c->pending.barrier = true;
    GridBarrier gb;
    gb.count = c->ws.barrier.as<unsigned int>();
    gb.err = reinterpret_cast<int *>(c->ws.barrier.as<unsigned int>() + 4);
    return gb;
}

// hole_filling (sources/gradientIBR.cu:87-152) on the device: hole list, then one persistent launch that runs
// the Jacobi iterations and their energy test (|change of the last channel's sum(lap * U)| < 1e-3).
static void hole_fill_async(lfrv_ctx *c, int W, int H, const uint8_t *vis, float *U, int max_iter) {
    Workspace &ws = c->ws;
    const size_t N = (size_t)W * H;
    cudaStream_t s = c->stream;
    ws.holes.ensure(sizeof(int) * (N + H + 16));
    ws.hole_count.ensure(sizeof(int) * 4);
    launch_hole_list(W, H, vis, ws.holes.as<int>(), ws.hole_count.as<int>(), s, c->launches);
    check_launch("hole list");
    ws.Ua.ensure(3 * N * sizeof(float));  // the grid-wide kernel's second buffer (it fills what it reads)
    double *part = partial_buf(c, 2 * (size_t)persistent_partials());
    const GridBarrier gb = fresh_barrier(c);
    LFRV_CUDA(launch_hole_fill_persistent(W, H, ws.holes.as<int>(), ws.hole_count.as<int>(), U, ws.Ua.as<float>(),
                                          part, gb, max_iter, solver_state(c) + 8, s, c->launches));
    c->pending.hole_fill = true;
}

// Sobel of every input view's luminance (compute_gradient, sources/gradientIBR_kernels.cuh:57-100).
static float *view_gradients(lfrv_ctx *c, const Geometry &G, const float *img, cudaStream_t st) {
    Workspace &ws = c->ws;
    ws.vgrad.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    float *vg = ws.vgrad.as<float>();
    launch_sobel(G.w, G.h, G.V, img, (size_t)3 * G.n, (size_t)G.n, vg, vg + G.n, (size_t)2 * G.n, nullptr, nullptr,
                 st, c->launches);
    check_launch("view sobel");
    return vg;
}

// BF16 views: their luminance Sobel into a BF16 stack (V x 2 x n), in the same workspace buffer.
static void *view_gradients_bf16(lfrv_ctx *c, const Geometry &G, const void *img, cudaStream_t st) {
    Workspace &ws = c->ws;
    ws.vgrad.ensure(sizeof(uint16_t) * 2 * (size_t)G.V * G.n);
    uint16_t *vg = ws.vgrad.as<uint16_t>();
    launch_view_sobel_bf16(G.w, G.h, G.V, img, (size_t)3 * G.n, (size_t)G.n, vg, vg + G.n, (size_t)2 * G.n, st,
                           c->launches);
    check_launch("view sobel (bf16)");
    return vg;
}

static void u_gradient(lfrv_ctx *c, const Geometry &G, const Buckets &B, const float *img, const float *tau2,
                       const float *wgt, float s2, float *gx, float *gy, float *mask) {
    float *vg = view_gradients(c, G, img, c->stream);
    launch_u_gradient(G, B, tau2, vg, wgt, s2, gx, gy, mask, c->stream, c->launches);
    check_launch("gradient splat");
}

// possion_conj_grad with the reference's loop (faithful, defect D1): 5 iterations, host-side scalars as the
// reference computes them (sources/solver.cu:612-676).
static int cg_faithful(lfrv_ctx *c, int W, int H, const float *gx, const float *gy, float *U,
                       double *trace = nullptr) {
    Workspace &ws = c->ws;
    const size_t N = (size_t)W * H;
    cudaStream_t s = c->stream;
    ws.r.ensure(3 * N * sizeof(float));
    ws.d.ensure(3 * N * sizeof(float));
    ws.q.ensure(3 * N * sizeof(float));
    float *r = ws.r.as<float>(), *d = ws.d.as<float>(), *q = ws.q.as<float>();
    const int np = cg_partials(W, H);
    double *part = partial_buf(c, 3 * (size_t)np);
    // energy trace: the quadratic energy of each iterate against the starting image u0
    const int trace_cap = trace ? c->pending.trace_cap : 0;
    if (trace) {
        ws.U0.ensure(3 * N * sizeof(float));
        LFRV_CUDA(cudaMemcpyAsync(ws.U0.p, U, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    ws.sums.ensure(sizeof(double) * 64);
    double *sums = ws.sums.as<double>();
    auto reduce3 = [&](double out[3]) {
        launch_reduce_segments(np, 3, part, sums, s, c->launches);
        check_launch("reduce3");
        LFRV_CUDA(cudaMemcpyAsync(out, sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
        sync(c);
    };
    const float lambda = 1.0f;  // possion_conj_grad: lambda = 1.0 (solver.cu:541)
    double delta[3];
    launch_cg_init(W, H, U, gx, gy, r, d, true, part, s, c->launches);
    check_launch("cg init");
    reduce3(delta);
    double dAlpha[3] = {0, 0, 0};
    const float beta[3] = {1.0f, 1.0f, 1.0f};
    int it;
    for (it = 0; it < 5; ++it) {
        double dq[3], rr[3];
        launch_cg_apply(W, H, d, lambda, q, part, s, c->launches);
        check_launch("cg apply");
        reduce3(dq);
        float alpha[3];
        for (int ch = 0; ch < 3; ++ch) {
            dAlpha[ch] += dq[ch];
            alpha[ch] = (float)delta[ch] / (float)dAlpha[ch];
        }
        launch_cg_update(W, H, alpha, d, q, U, r, part, s, c->launches);
        check_launch("cg update");
        reduce3(rr);
        for (int ch = 0; ch < 3; ++ch) dAlpha[ch] = (double)alpha[ch] + rr[ch];
        launch_cg_dir(W, H, beta, r, d, s, c->launches);
        check_launch("cg dir");
        if (it < trace_cap) {
            launch_cg_energy(W, H, U, ws.U0.as<float>(), gx, gy, part, s, c->launches);
            launch_reduce_final(np, part, trace + it, s, c->launches);
            check_launch("cg energy trace");
        }
    }
    return it;
}

// Corrected CG: one persistent launch (FP32 iterates, FP64 dot products, certified-gap stop on the device).
static void cg_persistent_async(lfrv_ctx *c, int W, int H, int max_iter, double gap_tol, const float *gx,
                                const float *gy, float *U, const float *U0 = nullptr, double *trace = nullptr,
                                int trace_cap = 0) {
    Workspace &ws = c->ws;
    const size_t N = (size_t)W * H;
    ws.r.ensure(3 * N * sizeof(float));
    ws.d.ensure(3 * N * sizeof(float));
    ws.q.ensure(3 * N * sizeof(float));
    const size_t np = (size_t)persistent_partials();
    double *part = partial_buf(c, 8 * np);
    const GridBarrier gb = fresh_barrier(c);
    LFRV_CUDA(launch_cg_persistent(W, H, gx, gy, U, ws.r.as<float>(), ws.d.as<float>(), ws.q.as<float>(), part,
                                   part + 4 * np, gb, max_iter, gap_tol, solver_state(c), c->stream, c->launches,
                                   U0, trace, trace_cap));
    c->pending.cg = true;
}

// IBR_gradient up to the CG (sources/gradientIBR.cpp:12-120): weights, the set-up pass (visibility, weighted
// average, gradient splat) into U, gx, gy, then hole filling of U (or U = init).
static void gradient_prepare(lfrv_ctx *c, const lfrv_config &cfg, const Geometry &G, const float *img,
                             const float *tau2, const float *dp2, const float *init, float *U, float *gx, float *gy,
                             void *learn_in = nullptr, cudaEvent_t views_ready = nullptr,
                             const void *vg_early = nullptr) {
    const size_t N = G.N;
    cudaStream_t s = c->stream;
    Workspace &ws = c->ws;
    const float s2 = cfg.sigma_sensor * cfg.sigma_sensor;
    ColorBuffers b = color_buffers(c, G);
    ws.mask.ensure(N * sizeof(float));
    // BF16 storage: img holds BF16 views, and the view gradients and weights are written in BF16
    const bool bf = cfg.bf16_storage != 0;
    // The weights and the view gradients depend only on tau, dp and the views: they run on the side stream
    // while the inverse map is built on the context stream, which waits for them before the set-up pass.
    // With per-kernel profiling on, everything stays on the context stream, so that each kernel's event time
    // is its own and not shared with a concurrent one; so it does in the helper lanes of a batched call, whose
    // streams already run beside each other.
    const bool fork = c->launches.prof == nullptr && !c->lane;
    cudaStream_t side = fork ? side_stream(c) : s;
    if (fork) {
        LFRV_CUDA(cudaEventRecord(c->side_fork, s));
        LFRV_CUDA(cudaStreamWaitEvent(side, c->side_fork, 0));
    }
    // compute_weights with U = 0 (sources/gradientIBR.cu:575-577): the unmasked Sobel of 0 is 0, so the
    // gathered gradient is 0 and the weights reduce to the deformation weights over sigma^2
    launch_weights(G, nullptr, nullptr, tau2, dp2, cfg.sigma_sensor, cfg.ugrad_threshold, b.wgt, side, c->launches,
                   bf);
    check_launch("weights");
    // views still uploading (views_ready): only the view gradients wait for them, and the set-up through the join.
    // vg_early: the caller already launched them on the side stream, ahead of the weights
    if (views_ready && !vg_early) LFRV_CUDA(cudaStreamWaitEvent(side, views_ready, 0));
    const void *vg = vg_early ? vg_early
                     : bf     ? view_gradients_bf16(c, G, img, side)
                              : (const void *)view_gradients(c, G, img, side);
    if (fork) LFRV_CUDA(cudaEventRecord(c->side_join, side));
    const Buckets B = build_buckets(c, G, tau2);
    if (fork) LFRV_CUDA(cudaStreamWaitEvent(s, c->side_join, 0));
    // visibility, weighted average and gradient splat in one pass of the inverse map
    launch_gradient_setup(G, B, tau2, img, vg, b.wgt, s2, b.vis, U, gx, gy, ws.mask.as<float>(), s, c->launches, bf);
    check_launch("gradient set-up");
    if (init) LFRV_CUDA(cudaMemcpyAsync(U, init, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    else hole_fill_async(c, G.W, G.H, b.vis, U, cfg.hole_fill_iter);
    // the learned warm start's input: the set-up products and the first views splatted one at a time
    if (learn_in) {
        launch_learn_input(G, B, tau2, img, b.wgt, U, gx, gy, b.vis, learn_in, s, c->launches, bf);
        check_launch("learned input");
    }
}

static void gradient_solve(lfrv_ctx *c, const lfrv_config &cfg, const float *img, const float *tau2, const float *dp2,
                           const float *init, float *out, lfrv_stats *st, cudaEvent_t views_ready = nullptr,
                           const void *vg_early = nullptr) {
    check_solver_options(cfg);
    const Geometry G = geometry(cfg);
    if (G.W < 2 || G.H < 2) raise(LFRV_E_ARG, "IBR_gradient needs a target of at least 2 x 2 pixels");
    const size_t N = G.N;
    cudaStream_t s = c->stream;
    Workspace &ws = c->ws;
    ColorBuffers b = color_buffers(c, G);
    float *U = ws.U.as<float>();
    c->pending = Pending{};
    double *trace = trace_request(c, st);
    gradient_prepare(c, cfg, G, img, tau2, dp2, init, U, b.gx, b.gy, nullptr, views_ready, vg_early);
    int it_faithful = 0;
    if (cfg.faithful) {
        it_faithful = cg_faithful(c, G.W, G.H, b.gx, b.gy, U, trace);
        if (trace) c->pending.trace_len = std::min(it_faithful, st->trace_capacity);
    } else {
        cg_persistent_async(c, G.W, G.H, cfg.cg_max_iter, cfg.cg_gap_tol, b.gx, b.gy, U, nullptr, trace,
                            trace ? st->trace_capacity : 0);
    }
    LFRV_CUDA(cudaMemcpyAsync(out, U, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, s));
    c->pending.stats = st;
    c->pending.gap_tol = cfg.cg_gap_tol;
    if (st) {
        st->outer_iterations = it_faithful;
        st->hole_fill_iterations = 0;
        st->gap = 0;
        st->stop_reason = 0;
    }
}

// After the stream has completed: solver statistics kept on the device, and the barrier status.
void finish_stats(lfrv_ctx *c) {
    Pending &p = c->pending;
    if (!p.cg && !p.hole_fill && !p.barrier && !p.trace_host) return;
    double state[16];
    int bar[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (p.cg || p.hole_fill) LFRV_CUDA(cudaMemcpy(state, c->ws.state.p, sizeof(state), cudaMemcpyDeviceToHost));
    if (p.barrier) LFRV_CUDA(cudaMemcpy(bar, c->ws.barrier.p, sizeof(bar), cudaMemcpyDeviceToHost));
    const bool timeout = bar[4] != 0;
    if (p.stats) {
        if (p.hole_fill) p.stats->hole_fill_iterations = (int)state[8];
        if (p.cg) {
            p.stats->outer_iterations = (int)state[5];
            p.stats->gap = state[4];
            p.stats->energy = state[3];
            p.stats->stop_reason = (p.gap_tol > 0 && state[4] <= p.gap_tol) ? 4 : 0;
        }
    }
    if (p.trace_host) {
        int len = p.trace_len >= 0 ? p.trace_len : (p.cg ? (int)state[5] : 0);
        len = std::max(0, std::min(len, p.trace_cap));
        if (len > 0)
            LFRV_CUDA(cudaMemcpy(p.trace_host, c->ws.trace.p, sizeof(double) * len, cudaMemcpyDeviceToHost));
        if (p.stats) p.stats->trace_length = len;
    }
    p = Pending{};
    if (timeout) raise(LFRV_E_TIMEOUT, "a device-side grid barrier gave up waiting (persistent solver)");
}

// ------------------------------------------------------------------ warp stage
static void mat3mul(const double *A, const double *B, double *C) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += A[3 * r + k] * B[3 * k + c];
            C[3 * r + c] = s;
        }
}

static void inv3(const double *m, double *o) {
    const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double det = a * A + b * B + c * C;
    if (det == 0) raise(LFRV_E_ARG, "singular camera intrinsics");
    o[0] = A / det;
    o[1] = -(b * i - c * h) / det;
    o[2] = (b * f - c * e) / det;
    o[3] = B / det;
    o[4] = (a * i - c * g) / det;
    o[5] = -(a * f - c * d) / det;
    o[6] = C / det;
    o[7] = -(a * h - b * g) / det;
    o[8] = (a * e - b * d) / det;
}

// Folds view k and target u into M = K_u R_u R_k^T K_k^-1, b = K_u (t_u - R_u R_k^T t_k).
static void fold_camera(const lfrv_camera &k, const lfrv_camera &u, float *Mout, float *bout) {
    double Kk[9], Rk[9], Ku[9], Ru[9], Kki[9], RkT[9];
    for (int i = 0; i < 9; ++i) {
        Kk[i] = k.K[i];
        Rk[i] = k.R[i];
        Ku[i] = u.K[i];
        Ru[i] = u.R[i];
    }
    inv3(Kk, Kki);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) RkT[3 * r + c] = Rk[3 * c + r];
    double T1[9], T2[9], M[9];
    mat3mul(RkT, Kki, T1);
    mat3mul(Ru, T1, T2);
    mat3mul(Ku, T2, M);
    double RuRkT[9];
    mat3mul(Ru, RkT, RuRkT);
    double v[3];
    for (int r = 0; r < 3; ++r) {
        double sacc = 0;
        for (int c = 0; c < 3; ++c) sacc += RuRkT[3 * r + c] * k.t[c];
        v[r] = u.t[r] - sacc;
    }
    for (int i = 0; i < 9; ++i) Mout[i] = (float)M[i];
    for (int r = 0; r < 3; ++r) {
        double sacc = 0;
        for (int c = 0; c < 3; ++c) sacc += Ku[3 * r + c] * v[c];
        bout[r] = (float)sacc;
    }
}

// Depth maps arriving in view chunks on the copy stream: chunk k (views up to v_end[k]) is complete when
// depth_ready[k] fires; the colour views when views_ready fires.
struct UploadPlan {
    int chunks = 0;
    int v_end[4] = {0, 0, 0, 0};
    cudaEvent_t depth_ready[4] = {};
    cudaEvent_t views_ready = nullptr;
};

static void warp(lfrv_ctx *c, int V, int w, int h, const float *depth, const lfrv_camera *cams,
                 const lfrv_camera *target, float *tau3, float *dpart3, float *tau2, float *dp2, float *zbuf_out,
                 const UploadPlan *plan = nullptr, const Geometry *count_for = nullptr) {
    if (V < 1 || V > kMaxViews || w <= 0 || h <= 0 || !depth || !cams || !target)
        raise(LFRV_E_ARG, "bad warp arguments");
    Workspace &ws = c->ws;
    const int W = target->width, H = target->height;
    if (W <= 0 || H <= 0) raise(LFRV_E_ARG, "bad target size");
    const size_t N = (size_t)W * H;
    // the folded cameras travel as a kernel parameter: no upload, no host synchronisation
    WarpCams wc;
    std::memset(&wc, 0, sizeof(wc));
    for (int v = 0; v < V; ++v) fold_camera(cams[v], *target, wc.M[v], wc.b[v]);
    ws.zkey.ensure(sizeof(unsigned long long) * N);
    ws.zbuf.ensure(sizeof(float) * N);
    ws.zdefer.ensure(sizeof(unsigned int) * zsplat_defer_words(V, w, h));
    launch_zbuffer_clear(W, H, ws.zkey.as<unsigned long long>(), c->stream, c->launches);
    // count_for (the solve's geometry, whose inverse map is built next from tau2): k_tau counts its buckets. The
    // counts are cleared here, ahead of the splat, so that k_tau directly follows the z-buffer kernels
    BucketCount bc;
    c->buckets_counted = false;
    if (count_for && tau2) {
        const Buckets B = bucket_buffers(c, *count_for);
        LFRV_CUDA(cudaMemsetAsync(B.count, 0, sizeof(unsigned int) * B.nb, c->stream));
        if (B.mask)
            LFRV_CUDA(cudaMemsetAsync(B.mask, 0, sizeof(unsigned long long) * B.nb * B.mask_words, c->stream));
        bc.count = B.count;
        bc.mask = B.mask;
        bc.dsf = count_for->dsf;
        bc.BW = B.BW;
        bc.nb = B.nb;
    }
    if (plan) {
        // splat each chunk of views as soon as its depth maps have arrived
        int v0 = 0;
        for (int k = 0; k < plan->chunks; ++k) {
            LFRV_CUDA(cudaStreamWaitEvent(c->stream, plan->depth_ready[k], 0));
            const int v1 = plan->v_end[k];
            WarpCams part;
            std::memset(&part, 0, sizeof(part));
            for (int v = v0; v < v1; ++v) {
                std::memcpy(part.M[v - v0], wc.M[v], sizeof(wc.M[v]));
                std::memcpy(part.b[v - v0], wc.b[v], sizeof(wc.b[v]));
            }
            launch_zbuffer_splat(v1 - v0, w, h, depth + (size_t)v0 * 3 * w * h, part, W, H,
                                 ws.zkey.as<unsigned long long>(), ws.zdefer.as<unsigned int>(), c->stream,
                                 c->launches);
            v0 = v1;
        }
    } else {
        launch_zbuffer_splat(V, w, h, depth, wc, W, H, ws.zkey.as<unsigned long long>(), ws.zdefer.as<unsigned int>(),
                             c->stream, c->launches);
    }
    // the resolved depth map only when the caller wants it; otherwise k_tau samples the keys themselves
    if (zbuf_out)
        launch_zbuffer_resolve(W, H, ws.zkey.as<unsigned long long>(), ws.zbuf.as<float>(), c->stream, c->launches);
    check_launch("z-buffer");
    launch_tau(V, w, h, depth, wc, W, H, zbuf_out ? ws.zbuf.as<float>() : nullptr, tau3, dpart3, tau2, dp2, c->stream,
               c->launches, bc.count ? &bc : nullptr, ws.zkey.as<unsigned long long>());
    check_launch("tau");
    if (bc.count) {
        c->buckets_counted = true;
        geometry_key(*count_for, c->counted_geometry);
        c->counted_tau = tau2;
    }
    if (zbuf_out)
        LFRV_CUDA(cudaMemcpyAsync(zbuf_out, ws.zbuf.p, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->stream));
}

// ------------------------------------------------------------------ helpers for host-buffer entry points
struct HostIO {
    lfrv_ctx *c;
    template <class T>
    T *up(DevBuf &buf, const T *host, size_t count) {
        if (!host) return nullptr;
        buf.ensure(sizeof(T) * count);
        LFRV_CUDA(cudaMemcpyAsync(buf.p, host, sizeof(T) * count, cudaMemcpyHostToDevice, c->stream));
        return buf.as<T>();
    }
    template <class T>
    void down(T *host, const T *dev, size_t count) {
        if (!host) return;
        LFRV_CUDA(cudaMemcpyAsync(host, dev, sizeof(T) * count, cudaMemcpyDeviceToHost, c->stream));
    }
};

// Converts caller tau (tau_channels per view) and dpart (3 per view) into the solver layout.
static void prepare_geometry_inputs(lfrv_ctx *c, const Geometry &G, const float *d_tau, int tau_channels,
                                    const float *d_dpart) {
    if (tau_channels != 2 && tau_channels != 3) raise(LFRV_E_ARG, "tau_channels must be 2 or 3");
    Workspace &ws = c->ws;
    ws.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    ws.dp.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    launch_copy_tau(G.V, G.n, d_tau, tau_channels, ws.tau.as<float>(), c->stream, c->launches);
    if (d_dpart) launch_premultiply_dpart(G.V, G.n, d_dpart, 3, ws.dp.as<float>(), c->stream, c->launches);
    else LFRV_CUDA(cudaMemsetAsync(ws.dp.p, 0, sizeof(float) * 2 * (size_t)G.V * G.n, c->stream));
    check_launch("input layout");
}

static void begin_timing(lfrv_ctx *c) {
    c->pending = Pending{};
    LFRV_CUDA(cudaEventRecord(c->ev0, c->stream));
}
static void end_timing(lfrv_ctx *c, lfrv_stats *st, long long launches0) {
    LFRV_CUDA(cudaEventRecord(c->ev1, c->stream));
    LFRV_CUDA(cudaEventSynchronize(c->ev1));
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        st->seconds = ms * 1e-3;
        st->kernel_launches = (int)(c->launches.n - launches0);
    }
    finish_stats(c);
}

}  // namespace lfrv

using namespace lfrv;

static cudaStream_t copy_stream(lfrv_ctx *c);

// (every call starts without counted buckets: a count the warp stage took belongs to the call that took it)
#define CTX_CHECK(ctx)                                                   \
    if (!(ctx)) return lfrv::fail(LFRV_E_ARG, "null context");           \
    LFRV_CUDA(cudaSetDevice((ctx)->device));                             \
    (ctx)->buckets_counted = false;

// ====================================================================== contexts
extern "C" int lfrv_ctx_create(lfrv_ctx **out, int device) {
    LFRV_API_BEGIN
    if (!out) return fail(LFRV_E_ARG, "null output pointer");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(LFRV_E_NODEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count) return fail(LFRV_E_ARG, "device %d out of range", device);
    LFRV_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    LFRV_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major * 10 + prop.minor < 100)
        return fail(LFRV_E_NODEVICE, "device %d is sm_%d%d; this library carries sm_103a code only", device,
                    prop.major, prop.minor);
    lfrv_ctx *c = new lfrv_ctx;
    c->device = device;
    LFRV_CUDA(cudaEventCreate(&c->ev0));
    LFRV_CUDA(cudaEventCreate(&c->ev1));
    LFRV_CUDA(cudaEventCreateWithFlags(&c->vg_ready, cudaEventDisableTiming));
    gaussian_kernel_init();
    {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            delete c;
            return fail(LFRV_E_NODEVICE, "kernel image not loadable on device %d: %s", device, cudaGetErrorString(e));
        }
    }
    *out = c;
    LFRV_API_END
}

extern "C" int lfrv_ctx_destroy(lfrv_ctx *ctx) {
    LFRV_API_BEGIN
    if (!ctx) return LFRV_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    else cudaDeviceSynchronize();
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->vg_ready) cudaEventDestroy(ctx->vg_ready);
    for (std::vector<lfrv_ctx *> *group : {&ctx->lanes, &ctx->tv_jobs})
        for (lfrv_ctx *l : *group) {
            cudaStreamSynchronize(l->stream);
            destroy_side_stream(l);
            cudaStreamDestroy(l->stream);
            if (l->host_sums) cudaFreeHost(l->host_sums);
            if (l->ev0) cudaEventDestroy(l->ev0);
            l->prof.destroy();
            delete l;
        }
    if (ctx->host_sums) cudaFreeHost(ctx->host_sums);
    destroy_side_stream(ctx);
    ctx->graph.reset({});
    for (cudaEvent_t e : ctx->lane_done) cudaEventDestroy(e);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
        cudaEventDestroy(ctx->up_start);
        cudaEventDestroy(ctx->up_views);
        cudaEventDestroy(ctx->out_ready);
        for (auto e : ctx->up_depth) cudaEventDestroy(e);
    }
    ctx->prof.destroy();
    delete ctx;
    LFRV_API_END
}

extern "C" int lfrv_ctx_set_stream(lfrv_ctx *ctx, void *cuda_stream) {
    LFRV_API_BEGIN
    if (!ctx) return fail(LFRV_E_ARG, "null context");
    ctx->stream = (cudaStream_t)cuda_stream;
    LFRV_API_END
}

extern "C" int lfrv_ctx_launch_count(lfrv_ctx *ctx, long long *count, int reset) {
    LFRV_API_BEGIN
    if (!ctx || !count) return fail(LFRV_E_ARG, "null argument");
    *count = ctx->launches.n;
    if (reset) ctx->launches.n = 0;
    LFRV_API_END
}

extern "C" int lfrv_ctx_profile(lfrv_ctx *ctx, int enable) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (enable) {
        ctx->prof.init(1 << 14);
        ctx->prof.reset();
        ctx->launches.prof = &ctx->prof;
    } else {
        ctx->launches.prof = nullptr;
    }
    LFRV_API_END
}

extern "C" int lfrv_ctx_profile_read(lfrv_ctx *ctx, int index, char *name, size_t name_len, double *total_ms,
                                     long long *launches) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    ctx->prof.fold();
    const KernelProfiler &p = ctx->prof;
    if (index < 0 || index >= (int)p.names.size()) return fail(LFRV_E_ARG, "profile index %d out of range", index);
    if (name && name_len) std::snprintf(name, name_len, "%s", p.names[index].c_str());
    if (total_ms) *total_ms = p.ms[index];
    if (launches) *launches = p.count[index];
    LFRV_API_END
}

// ====================================================================== warp
extern "C" int lfrv_warp_dev(lfrv_ctx *ctx, int nviews, int w, int h, const float *d_depth, const lfrv_camera *cams,
                             const lfrv_camera *target, float *d_tau, float *d_dpart, float *d_zbuf) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    warp(ctx, nviews, w, h, d_depth, cams, target, d_tau, d_dpart, nullptr, nullptr, d_zbuf);
    LFRV_API_END
}

// Float camera record of the warps-from-depth kernels, computed as the reference's glm float arithmetic.
static void wfd_camera(const lfrv_camera &c, float *o) {
    o[0] = c.K[0];
    o[1] = c.K[4];
    o[2] = c.K[2];
    o[3] = c.K[5];
    for (int i = 0; i < 9; ++i) o[4 + i] = c.R[i];
    for (int r = 0; r < 3; ++r) o[13 + r] = -(c.R[0 * 3 + r] * c.t[0] + c.R[1 * 3 + r] * c.t[1] + c.R[2 * 3 + r] * c.t[2]);
    for (int r = 0; r < 3; ++r) {
        for (int col = 0; col < 3; ++col)
            o[16 + r * 4 + col] =
                c.K[r * 3 + 0] * c.R[0 * 3 + col] + c.K[r * 3 + 1] * c.R[1 * 3 + col] + c.K[r * 3 + 2] * c.R[2 * 3 + col];
        o[16 + r * 4 + 3] = c.K[r * 3 + 0] * c.t[0] + c.K[r * 3 + 1] * c.t[1] + c.K[r * 3 + 2] * c.t[2];
    }
}

// import_warps_from_depth (sources/import.cpp:243-450) on device buffers.
static void warp_from_depth(lfrv_ctx *c, int nviews, int w, int h, int dsf, const float *d_depth, int depth_channels,
                            const lfrv_camera *cams, const lfrv_camera *target, int faithful, float *d_tau) {
    if (nviews < 1 || nviews > kMaxViews || w <= 0 || h <= 0 || dsf < 1 || !d_depth || !cams || !target || !d_tau ||
        depth_channels < 1)
        raise(LFRV_E_ARG, "bad warp-from-depth arguments");
    const int W = target->width, H = target->height;
    if (W <= 0 || H <= 0) raise(LFRV_E_ARG, "bad target size");
    for (int v = 0; v <= nviews; ++v) {
        const lfrv_camera &k = v < nviews ? cams[v] : *target;
        if (k.K[0] == 0.0f || k.K[4] == 0.0f) raise(LFRV_E_ARG, "camera %d: zero focal length", v);
    }
    WfdCams wc;
    std::memset(&wc, 0, sizeof(wc));
    for (int v = 0; v < nviews; ++v) wfd_camera(cams[v], wc.c[v]);
    wfd_camera(*target, wc.c[nviews]);
    c->ws.ukey.ensure(sizeof(unsigned int) * (size_t)W * H);
    launch_warp_from_depth(nviews, w, h, dsf, d_depth, depth_channels, wc, W, H, faithful, c->ws.ukey.as<unsigned int>(),
                           d_tau, c->stream, c->launches);
    check_launch("warp from depth");
}

extern "C" int lfrv_warp_from_depth_dev(lfrv_ctx *ctx, int nviews, int w, int h, int dsf, const float *d_depth,
                                        int depth_channels, const lfrv_camera *cams, const lfrv_camera *target,
                                        int faithful, float *d_tau) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    warp_from_depth(ctx, nviews, w, h, dsf, d_depth, depth_channels, cams, target, faithful, d_tau);
    LFRV_API_END
}

extern "C" int lfrv_warp_from_depth(lfrv_ctx *ctx, int nviews, int w, int h, int dsf, const float *depth,
                                    int depth_channels, const lfrv_camera *cams, const lfrv_camera *target,
                                    int faithful, float *tau) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!depth || !tau || nviews < 1 || depth_channels < 1) return fail(LFRV_E_ARG, "bad arguments");
    const size_t n = (size_t)w * h;
    HostIO io{ctx};
    const float *dd = io.up(ctx->ws.depth, depth, (size_t)nviews * depth_channels * n);
    ctx->ws.in_tau.ensure(sizeof(float) * 3 * nviews * n);
    warp_from_depth(ctx, nviews, w, h, dsf, dd, depth_channels, cams, target, faithful, ctx->ws.in_tau.as<float>());
    io.down(tau, ctx->ws.in_tau.as<float>(), 3 * (size_t)nviews * n);
    sync(ctx);
    LFRV_API_END
}

// fromRadial2Ortho.frag (sources/openGL/frameBuffer.cpp:263-300, run by InputView::filterDepthmap,
// sources/openGL/view.cpp:723-733) on device depth maps, in place.
static void radial_to_ortho(lfrv_ctx *c, int nviews, int w, int h, const lfrv_camera *cams, float *d_depth) {
    if (nviews < 1 || nviews > kMaxViews || w <= 0 || h <= 0 || !cams || !d_depth)
        raise(LFRV_E_ARG, "bad radial-to-ortho arguments");
    WarpCams kinv;
    std::memset(&kinv, 0, sizeof(kinv));
    for (int v = 0; v < nviews; ++v) {
        const float *K = cams[v].K;
        double m[9], inv[9];
        for (int i = 0; i < 9; ++i) m[i] = K[i];
        const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                           m[2] * (m[3] * m[7] - m[4] * m[6]);
        if (det == 0.0) raise(LFRV_E_ARG, "camera %d: singular K", v);
        inv[0] = (m[4] * m[8] - m[5] * m[7]) / det;
        inv[1] = (m[2] * m[7] - m[1] * m[8]) / det;
        inv[2] = (m[1] * m[5] - m[2] * m[4]) / det;
        inv[3] = (m[5] * m[6] - m[3] * m[8]) / det;
        inv[4] = (m[0] * m[8] - m[2] * m[6]) / det;
        inv[5] = (m[2] * m[3] - m[0] * m[5]) / det;
        inv[6] = (m[3] * m[7] - m[4] * m[6]) / det;
        inv[7] = (m[1] * m[6] - m[0] * m[7]) / det;
        inv[8] = (m[0] * m[4] - m[1] * m[3]) / det;
        for (int i = 0; i < 9; ++i) kinv.M[v][i] = (float)inv[i];
    }
    launch_radial_to_ortho(nviews, w, h, kinv, d_depth, c->stream, c->launches);
    check_launch("radial to ortho");
}

extern "C" int lfrv_depth_radial_to_ortho_dev(lfrv_ctx *ctx, int nviews, int w, int h, const lfrv_camera *cams,
                                              float *d_depth) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    radial_to_ortho(ctx, nviews, w, h, cams, d_depth);
    LFRV_API_END
}

extern "C" int lfrv_depth_radial_to_ortho(lfrv_ctx *ctx, int nviews, int w, int h, const lfrv_camera *cams,
                                          float *depth) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!depth) return fail(LFRV_E_ARG, "null depth");
    const size_t count = (size_t)nviews * 3 * (size_t)w * h;
    HostIO io{ctx};
    float *d = io.up(ctx->ws.depth, depth, count);
    radial_to_ortho(ctx, nviews, w, h, cams, d);
    io.down(depth, d, count);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_warp(lfrv_ctx *ctx, int nviews, int w, int h, const float *depth, const lfrv_camera *cams,
                         const lfrv_camera *target, float *tau, float *dpart, float *zbuf) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!depth || !target) return fail(LFRV_E_ARG, "null argument");
    HostIO io{ctx};
    const size_t n = (size_t)w * h, V = (size_t)nviews, N = (size_t)target->width * target->height;
    float *dd = io.up(ctx->ws.depth, depth, V * 3 * n);
    ctx->ws.in_tau.ensure(sizeof(float) * V * 3 * n);
    ctx->ws.in_dpart.ensure(sizeof(float) * V * 3 * n);
    ctx->ws.out_img.ensure(sizeof(float) * N);
    warp(ctx, nviews, w, h, dd, cams, target, ctx->ws.in_tau.as<float>(), ctx->ws.in_dpart.as<float>(), nullptr,
         nullptr, ctx->ws.out_img.as<float>());
    io.down(tau, ctx->ws.in_tau.as<float>(), V * 3 * n);
    io.down(dpart, ctx->ws.in_dpart.as<float>(), V * 3 * n);
    io.down(zbuf, ctx->ws.out_img.as<float>(), N);
    sync(ctx);
    LFRV_API_END
}

// ====================================================================== solvers
static int solve_dev(lfrv_ctx *ctx, const lfrv_config *cfg, bool color, const float *d_views, const float *d_tau,
                     int tau_channels, const float *d_dpart, const float *d_init, float *d_out, lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!cfg || !d_views || !d_tau || !d_out) return fail(LFRV_E_ARG, "null argument");
    reset_stats(stats);
    const Geometry G = geometry(*cfg);
    const long long l0 = ctx->launches.n;
    begin_timing(ctx);
    prepare_geometry_inputs(ctx, G, d_tau, tau_channels, d_dpart);
    if (color)
        color_solve(ctx, *cfg, d_views, ctx->ws.tau.as<float>(), ctx->ws.dp.as<float>(), d_init, d_out, stats);
    else
        gradient_solve(ctx, *cfg, d_views, ctx->ws.tau.as<float>(), ctx->ws.dp.as<float>(), d_init, d_out, stats);
    end_timing(ctx, stats, l0);
    LFRV_API_END
}

static int solve_host(lfrv_ctx *ctx, const lfrv_config *cfg, bool color, const float *views, const float *tau,
                      int tau_channels, const float *dpart, const float *init, float *out, lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!cfg || !views || !tau || !out) return fail(LFRV_E_ARG, "null argument");
    if (cfg->bf16_storage) return fail(LFRV_E_ARG, "bf16_storage needs device views (the *_dev entry points)");
    const Geometry G = geometry(*cfg);
    HostIO io{ctx};
    const size_t n = G.n, V = G.V;
    const float *dv = io.up(ctx->ws.in_views, views, V * 3 * n);
    const float *dt = io.up(ctx->ws.in_tau, tau, V * (size_t)tau_channels * n);
    const float *dd = io.up(ctx->ws.in_dpart, dpart, V * 3 * n);
    const float *di = io.up(ctx->ws.in_init, init, 3 * G.N);
    ctx->ws.out_img.ensure(sizeof(float) * 3 * G.N);
    const int rc = solve_dev(ctx, cfg, color, dv, dt, tau_channels, dd, di, ctx->ws.out_img.as<float>(), stats);
    if (rc != LFRV_OK) return rc;
    io.down(out, ctx->ws.out_img.as<float>(), 3 * G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_ibr_color_dev(lfrv_ctx *ctx, const lfrv_config *cfg, const float *d_views, const float *d_tau,
                                  int tau_channels, const float *d_dpart, const float *d_init, float *d_out,
                                  lfrv_stats *stats) {
    return solve_dev(ctx, cfg, true, d_views, d_tau, tau_channels, d_dpart, d_init, d_out, stats);
}
extern "C" int lfrv_ibr_gradient_dev(lfrv_ctx *ctx, const lfrv_config *cfg, const float *d_views, const float *d_tau,
                                     int tau_channels, const float *d_dpart, const float *d_init, float *d_out,
                                     lfrv_stats *stats) {
    return solve_dev(ctx, cfg, false, d_views, d_tau, tau_channels, d_dpart, d_init, d_out, stats);
}
extern "C" int lfrv_ibr_color(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                              int tau_channels, const float *dpart, const float *init, float *out, lfrv_stats *stats) {
    return solve_host(ctx, cfg, true, views, tau, tau_channels, dpart, init, out, stats);
}
extern "C" int lfrv_ibr_gradient(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                                 int tau_channels, const float *dpart, const float *init, float *out,
                                 lfrv_stats *stats) {
    return solve_host(ctx, cfg, false, views, tau, tau_channels, dpart, init, out, stats);
}

// Warp stage + solve of one target view on device buffers; with a plan the inputs are still arriving on the
// copy stream, and with host_out the result is copied back before the call synchronises.
// The stream work of one render call (between the call's timing events).
static void render_view_body(lfrv_ctx *ctx, const lfrv_config &cfg, int algorithm, const float *d_views,
                             const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target, float *d_out,
                             lfrv_stats *stats, const UploadPlan *plan, float *host_out) {
    const Geometry G = geometry(cfg);
    Workspace &ws = ctx->ws;
    ws.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    ws.dp.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    // IBR_gradient uses dtau/dz only in its weights, multiplied by the gradient of U = 0 (compute_weights with
    // U = 0): the warp stage does not write it and the weights take it as 0 (the same weights wherever they are
    // read: a pixel whose dtau/dz is not finite is outside the view and in no bucket)
    float *dp2 = algorithm == 0 ? ws.dp.as<float>() : nullptr;
    // IBR_gradient from device-resident views: their Sobel needs only the views, so it starts on the side stream
    // beside the warp stage (gradient_prepare's join after the weights also covers it). Not with per-kernel
    // profiling or in a helper lane, where gradient_prepare keeps its work on one stream.
    const void *vg_early = nullptr;
    if (algorithm == 1 && !plan && ctx->launches.prof == nullptr && !ctx->lane) {
        cudaStream_t side = side_stream(ctx);
        LFRV_CUDA(cudaEventRecord(ctx->side_fork, ctx->stream));
        LFRV_CUDA(cudaStreamWaitEvent(side, ctx->side_fork, 0));
        vg_early = cfg.bf16_storage ? view_gradients_bf16(ctx, G, d_views, side)
                                    : (const void *)view_gradients(ctx, G, d_views, side);
    }
    warp(ctx, G.V, G.w, G.h, d_depth, cams, target, nullptr, nullptr, ws.tau.as<float>(), dp2, nullptr, plan, &G);
    if (algorithm == 0) {
        if (plan) LFRV_CUDA(cudaStreamWaitEvent(ctx->stream, plan->views_ready, 0));
        color_solve(ctx, cfg, d_views, ws.tau.as<float>(), dp2, nullptr, d_out, stats);
    } else {
        // the inverse map and the weights need only the warps: they do not wait for the colour views' upload
        gradient_solve(ctx, cfg, d_views, ws.tau.as<float>(), nullptr, nullptr, d_out, stats,
                       plan ? plan->views_ready : nullptr, vg_early);
    }
    if (host_out)
        LFRV_CUDA(cudaMemcpyAsync(host_out, d_out, sizeof(float) * 3 * G.N, cudaMemcpyDeviceToHost, ctx->stream));
}

static void render_view_impl(lfrv_ctx *ctx, const lfrv_config &cfg, int algorithm, const float *d_views,
                             const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target, float *d_out,
                             lfrv_stats *stats, const UploadPlan *plan, float *host_out) {
    reset_stats(stats);
    const Geometry G = geometry(cfg);
    if (target->width != G.W || target->height != G.H) raise(LFRV_E_ARG, "target size mismatch");
    const long long l0 = ctx->launches.n;
    begin_timing(ctx);
    render_view_body(ctx, cfg, algorithm, d_views, d_depth, cams, target, d_out, stats, plan, host_out);
    end_timing(ctx, stats, l0);
}

// Repeated render calls through a CUDA graph. A call whose key (its arguments: config, pointers, cameras,
// target, stream) repeats the previous call's is captured once, the second time it is seen (the first run
// allocated its workspace), and replayed from then on: one graph launch instead of the ~25 launches, memsets,
// copies and events of the call, so the device does not idle while the host enqueues them. Only IBR_gradient
// with the corrected CG qualifies (no host synchronisation inside the call), and not while per-kernel profiling
// is on. The host state the call leaves (pending solver statistics, launch count) is recorded at capture and
// restored at each replay; any workspace reallocation since the capture invalidates the graph. body() enqueues
// the call's stream work. Returns false when the call must run uncaptured.
template <class Body>
static bool render_graph(lfrv_ctx *ctx, std::vector<unsigned char> key, lfrv_stats *stats, Body body) {
    RenderGraph &g = ctx->graph;
    if (g.key != key) {
        g.reset(std::move(key));
        g.seen = true;
        return false;
    }
    if (g.failed) return false;
    if (g.exec && g.epoch != g_alloc_epoch) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        return false;  // rerun uncaptured; the next identical call captures again
    }
    if (!g.exec) {
        const unsigned long long e0 = g_alloc_epoch;
        const long long l0 = ctx->launches.n;
        ctx->pending = Pending{};
        cudaGraph_t graph = nullptr;
        bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
        if (ok) {
            try {
                body();
            } catch (...) {
                ok = false;
            }
            ok = cudaStreamEndCapture(ctx->stream, &graph) == cudaSuccess && ok && graph && e0 == g_alloc_epoch;
            if (ok) ok = cudaGraphInstantiate(&g.exec, graph, 0) == cudaSuccess;
        }
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();  // a failed capture leaves its error here; the call reruns uncaptured
        if (!ok) {
            g.exec = nullptr;
            g.failed = true;
            ctx->launches.n = l0;
            ctx->pending = Pending{};
            return false;
        }
        g.epoch = e0;
        g.pending = ctx->pending;
        g.pending.stats = nullptr;
        g.launches = ctx->launches.n - l0;
        ctx->launches.n = l0;
    }
    reset_stats(stats);
    const long long l0 = ctx->launches.n;
    begin_timing(ctx);
    LFRV_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
    ctx->launches.n += g.launches;
    ctx->pending = g.pending;
    ctx->pending.stats = stats;
    end_timing(ctx, stats, l0);
    return true;
}

// The key of a render call: its argument bytes.
static std::vector<unsigned char> render_key(lfrv_ctx *ctx, const lfrv_config &cfg, int algorithm, const void *views,
                                             const void *depth, const void *out, const lfrv_camera *cams,
                                             const lfrv_camera *target) {
    std::vector<unsigned char> key;
    auto put = [&](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        key.insert(key.end(), c, c + n);
    };
    put(&cfg, sizeof(cfg));
    put(&algorithm, sizeof(algorithm));
    put(&views, sizeof(views));
    put(&depth, sizeof(depth));
    put(&out, sizeof(out));
    put(cams, sizeof(lfrv_camera) * (size_t)cfg.nviews);
    put(target, sizeof(*target));
    put(&ctx->stream, sizeof(ctx->stream));
    return key;
}

static bool graph_eligible(lfrv_ctx *ctx, const lfrv_config &cfg, int algorithm, const lfrv_camera *target,
                           const lfrv_stats *stats) {
    if (algorithm != 1 || cfg.faithful || ctx->launches.prof) return false;
    if (stats && stats->energy_trace && stats->trace_capacity > 0) return false;  // traced calls run uncaptured
    const Geometry G = geometry(cfg);
    return target->width == G.W && target->height == G.H;
}

extern "C" int lfrv_render_view_dev(lfrv_ctx *ctx, const lfrv_config *cfg, int algorithm, const float *d_views,
                                    const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target,
                                    float *d_out, lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!cfg || !d_views || !d_depth || !cams || !target || !d_out) return fail(LFRV_E_ARG, "null argument");
    const bool replayed =
        graph_eligible(ctx, *cfg, algorithm, target, stats) &&
        render_graph(ctx, render_key(ctx, *cfg, algorithm, d_views, d_depth, d_out, cams, target), stats, [&] {
            render_view_body(ctx, *cfg, algorithm, d_views, d_depth, cams, target, d_out, nullptr, nullptr, nullptr);
        });
    if (!replayed)
        render_view_impl(ctx, *cfg, algorithm, d_views, d_depth, cams, target, d_out, stats, nullptr, nullptr);
    LFRV_API_END
}

namespace lfrv {
void warmstart_predict_async(lfrv_warmstart *net, int H, int W, const void *d_input, const float *d_u0, float *d_pred);
void warmstart_check(lfrv_warmstart *net);
lfrv_ctx *warmstart_ctx(lfrv_warmstart *net);
}  // namespace lfrv

// ====================================================================== learned warm start
// Training data and warm-started solves of IBR_gradient with the corrected CG. The network sees the set-up
// products (anchor u0, gx, gy, visibility) and the first views splatted one at a time; its prediction only seeds
// the CG iterate, while the anchor u0 keeps the problem, its energy and the certified-gap stop unchanged.

static Geometry warm_geometry(const lfrv_config &cfg, const lfrv_camera *target) {
    if (cfg.faithful) raise(LFRV_E_ARG, "the learned warm start seeds the corrected CG (faithful = 0)");
    check_solver_options(cfg);
    const Geometry G = geometry(cfg);
    if (target->width != G.W || target->height != G.H) raise(LFRV_E_ARG, "target size mismatch");
    if (G.W % 8 || G.H % 8 || G.W < 8 || G.H < 8)
        raise(LFRV_E_ARG, "the learned warm start needs a target of multiples of 8 pixels (got %d x %d)", G.W, G.H);
    return G;
}

static void warm_features(lfrv_ctx *ctx, const lfrv_config &cfg, const float *d_views, const float *d_depth,
                          const lfrv_camera *cams, const lfrv_camera *target, void *d_input, float *d_u0,
                          float *d_solution, lfrv_stats *stats) {
    reset_stats(stats);
    const Geometry G = warm_geometry(cfg, target);
    const long long l0 = ctx->launches.n;
    begin_timing(ctx);
    Workspace &ws = ctx->ws;
    ws.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    // no dtau/dz: IBR_gradient's weights multiply it by the gradient of U = 0 (as in lfrv_render_view_dev)
    warp(ctx, G.V, G.w, G.h, d_depth, cams, target, nullptr, nullptr, ws.tau.as<float>(), nullptr, nullptr, nullptr, &G);
    ColorBuffers b = color_buffers(ctx, G);
    float *U = ws.U.as<float>();
    ctx->pending = Pending{};
    gradient_prepare(ctx, cfg, G, d_views, ws.tau.as<float>(), nullptr, nullptr, U, b.gx, b.gy, d_input);
    if (d_u0) LFRV_CUDA(cudaMemcpyAsync(d_u0, U, 3 * G.N * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    if (d_solution) {
        cg_persistent_async(ctx, G.W, G.H, cfg.cg_max_iter, cfg.cg_gap_tol, b.gx, b.gy, U);
        LFRV_CUDA(cudaMemcpyAsync(d_solution, U, 3 * G.N * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ctx->pending.stats = stats;
    ctx->pending.gap_tol = cfg.cg_gap_tol;
    end_timing(ctx, stats, l0);
}

static void render_view_warm(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_config &cfg, const float *d_views,
                             const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target, float *d_out,
                             lfrv_stats *stats) {
    reset_stats(stats);
    const Geometry G = warm_geometry(cfg, target);
    const long long l0 = ctx->launches.n;
    begin_timing(ctx);
    Workspace &ws = ctx->ws;
    ws.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
    ws.learn_in.ensure(G.N * kLearnChannels * 2);
    ws.seed.ensure(3 * G.N * sizeof(float));
    warp(ctx, G.V, G.w, G.h, d_depth, cams, target, nullptr, nullptr, ws.tau.as<float>(), nullptr, nullptr, nullptr, &G);
    ColorBuffers b = color_buffers(ctx, G);
    float *U = ws.U.as<float>(), *X = ws.seed.as<float>();
    ctx->pending = Pending{};
    gradient_prepare(ctx, cfg, G, d_views, ws.tau.as<float>(), nullptr, nullptr, U, b.gx, b.gy, ws.learn_in.p);
    warmstart_predict_async(net, G.H, G.W, ws.learn_in.p, U, X);
    cg_persistent_async(ctx, G.W, G.H, cfg.cg_max_iter, cfg.cg_gap_tol, b.gx, b.gy, X, U);
    LFRV_CUDA(cudaMemcpyAsync(d_out, X, 3 * G.N * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->pending.stats = stats;
    ctx->pending.gap_tol = cfg.cg_gap_tol;
    end_timing(ctx, stats, l0);
    warmstart_check(net);
}

extern "C" int lfrv_warmstart_features_dev(lfrv_ctx *ctx, const lfrv_config *cfg, const float *d_views,
                                           const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target,
                                           void *d_input, float *d_u0, float *d_solution, lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!cfg || !d_views || !d_depth || !cams || !target || !d_input) return fail(LFRV_E_ARG, "null argument");
    warm_features(ctx, *cfg, d_views, d_depth, cams, target, d_input, d_u0, d_solution, stats);
    LFRV_API_END
}

extern "C" int lfrv_render_view_warm_dev(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_config *cfg,
                                         const float *d_views, const float *d_depth, const lfrv_camera *cams,
                                         const lfrv_camera *target, float *d_out, lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!net || !cfg || !d_views || !d_depth || !cams || !target || !d_out) return fail(LFRV_E_ARG, "null argument");
    render_view_warm(ctx, net, *cfg, d_views, d_depth, cams, target, d_out, stats);
    LFRV_API_END
}

// ====================================================================== batched targets
// IBR_gradient jobs with the corrected CG share one k_cg_batch launch (per launch at most as many jobs as resident
// blocks); every other job runs on its own. Per gradient job the batch pool holds U, gx, gy, r, dA, dB (14 N
// floats) and 8 doubles of state.
// Host-buffer calls pass host_out (per job: a pinned host destination, or nullptr) and sent (per job, zeroed): an
// IBR_gradient job's output is then copied to host_out as soon as its CG is done, on the copy stream, while the next
// jobs run, and sent[job] is set. views_ready (or nullptr): an event the jobs wait for before they read their colour
// views (the warp stage reads only the depth maps, so it may start while the views are still being uploaded).
static void render_views(lfrv_ctx *c, const lfrv_view_job *jobs, int count, lfrv_warmstart *net = nullptr,
                         float *const *host_out = nullptr, char *sent = nullptr, cudaEvent_t views_ready = nullptr) {
    if (count <= 0 || !jobs) raise(LFRV_E_ARG, "empty batch");
    cudaStream_t s = c->stream;
    Workspace &ws = c->ws;
    struct Slot {
        int job;
        Geometry G;
        size_t off;  // float offset of the job's buffers in the pool
        bool seeded;  // the learned warm start seeds its CG (seed at 14 N + 16, network input after it)
    };
    if (net && warmstart_ctx(net) != c) raise(LFRV_E_ARG, "the warm-start network belongs to another context");
    std::vector<Slot> batched;
    // corrected IBR_color jobs with one meta iteration: each on a context of its own, advanced in lockstep
    std::vector<int> tv_idx;
    size_t pool = 0;
    for (int j = 0; j < count; ++j) {
        const lfrv_view_job &J = jobs[j];
        if (!J.cfg || !J.d_views || !J.d_depth || !J.cams || !J.target || !J.d_out)
            raise(LFRV_E_ARG, "job %d: null argument", j);
        const Geometry G = geometry(*J.cfg);
        if (J.target->width != G.W || J.target->height != G.H) raise(LFRV_E_ARG, "job %d: target size mismatch", j);
        reset_stats(J.stats);
        if (J.algorithm == 0 && !J.cfg->faithful && J.cfg->nmeta_iter == 1) tv_idx.push_back(j);
        if (J.algorithm == 1 && !J.cfg->faithful) {
            check_solver_options(*J.cfg);
            if (G.W < 2 || G.H < 2) raise(LFRV_E_ARG, "job %d: target smaller than 2 x 2", j);
            const bool seeded = net && G.W % 8 == 0 && G.H % 8 == 0;
            batched.push_back({j, G, pool, seeded});
            pool += 14 * G.N + 16;  // + 8 doubles of state, kept 64-byte aligned by the 16-float pad
            if (seeded) pool += 3 * G.N + (G.N * kLearnChannels * 2 + 63) / 64 * 16;  // seed + BF16 input
        }
    }
    ws.batch.ensure(sizeof(float) * std::max<size_t>(pool, 16));
    float *base = ws.batch.as<float>();
    c->pending = Pending{};
    // the batched jobs' warp stage, set-up and hole filling run on helper contexts (own stream and workspace
    // each, round robin), so that small targets overlap; the context stream waits for all of them. Four lanes,
    // or two when a target has 2^21 pixels or more: each of its kernels fills the GPU alone, and more streams
    // only share the L2 between more working sets (measured on 2048^2 targets of 80 views)
    size_t largest = 0;
    for (const Slot &sl : batched) largest = std::max(largest, sl.G.N);
    const int kLanes = largest >= ((size_t)1 << 21) ? 2 : 4;
    while ((int)c->lanes.size() < kLanes) {
        lfrv_ctx *l = new lfrv_ctx;
        l->device = c->device;
        LFRV_CUDA(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking));
        l->owns_stream = true;
        l->lane = true;
        c->lanes.push_back(l);
        cudaEvent_t e;
        LFRV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->lane_done.push_back(e);
    }
    LFRV_CUDA(cudaEventRecord(c->ev0, s));  // lanes start after what the caller queued on the context stream
    for (size_t k = 0; k < c->lanes.size(); ++k) {  // every lane (an earlier call may have used more)
        lfrv_ctx *l = c->lanes[k];
        l->launches.n = 0;
        l->launches.prof = nullptr;  // the profiler folds events per stream; lane kernels are counted, not timed
        l->pending = Pending{};
        if ((int)k < kLanes) LFRV_CUDA(cudaStreamWaitEvent(l->stream, c->ev0, 0));
    }
    // the corrected IBR_color jobs: warp stage and set-up on their own contexts (streams), up to the first step
    while (c->tv_jobs.size() < tv_idx.size()) {
        lfrv_ctx *l = new lfrv_ctx;
        l->device = c->device;
        LFRV_CUDA(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking));
        l->owns_stream = true;
        l->lane = true;
        c->tv_jobs.push_back(l);
    }
    std::vector<TvSolve> tv(tv_idx.size());
    for (size_t q = 0; q < tv_idx.size(); ++q) {
        const lfrv_view_job &J = jobs[tv_idx[q]];
        lfrv_ctx *l = c->tv_jobs[q];
        l->launches.n = 0;
        l->launches.prof = nullptr;
        l->pending = Pending{};
        LFRV_CUDA(cudaStreamWaitEvent(l->stream, c->ev0, 0));
        const Geometry G = geometry(*J.cfg);
        l->ws.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
        l->ws.dp.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
        warp(l, G.V, G.w, G.h, J.d_depth, J.cams, J.target, nullptr, nullptr, l->ws.tau.as<float>(),
             l->ws.dp.as<float>(), nullptr);
        if (views_ready) LFRV_CUDA(cudaStreamWaitEvent(l->stream, views_ready, 0));
        color_solve(l, *J.cfg, J.d_views, l->ws.tau.as<float>(), l->ws.dp.as<float>(), nullptr, J.d_out, J.stats,
                    &tv[q]);
        l->pending.trace_host = nullptr;  // the solve writes its trace from the host
    }
    // the view gradients (luminance Sobel of every view) depend only on the views: computed once per distinct light
    // field of the batched jobs, on the context stream while the lanes run the warp stage, and joined by event
    // before each job's set-up (targets that share a light field share them)
    struct VgField {
        const void *views;
        int V, w, h;
        bool bf;
        size_t off;
    };
    std::vector<VgField> fields;
    std::vector<size_t> vg_off(batched.size(), 0);
    size_t vg_bytes = 0;
    for (size_t q = 0; q < batched.size(); ++q) {
        const Slot &sl = batched[q];
        const lfrv_view_job &J = jobs[sl.job];
        const bool bf = J.cfg->bf16_storage != 0;
        size_t f = 0;
        while (f < fields.size() && !(fields[f].views == (const void *)J.d_views && fields[f].V == sl.G.V &&
                                      fields[f].w == sl.G.w && fields[f].h == sl.G.h && fields[f].bf == bf))
            ++f;
        if (f == fields.size()) {
            fields.push_back({J.d_views, sl.G.V, sl.G.w, sl.G.h, bf, vg_bytes});
            vg_bytes += (2 * (size_t)sl.G.V * sl.G.n * (bf ? 2 : 4) + 255) / 256 * 256;
        }
        vg_off[q] = fields[f].off;
    }
    if (!fields.empty()) {
        ws.vg_pool.ensure(vg_bytes);
        if (views_ready) LFRV_CUDA(cudaStreamWaitEvent(s, views_ready, 0));
        for (const VgField &f : fields) {
            const size_t n = (size_t)f.w * f.h;
            if (f.bf) {
                uint16_t *vg = reinterpret_cast<uint16_t *>(ws.vg_pool.as<char>() + f.off);
                launch_view_sobel_bf16(f.w, f.h, f.V, f.views, 3 * n, n, vg, vg + n, 2 * n, s, c->launches);
            } else {
                float *vg = reinterpret_cast<float *>(ws.vg_pool.as<char>() + f.off);
                launch_sobel(f.w, f.h, f.V, static_cast<const float *>(f.views), 3 * n, n, vg, vg + n, 2 * n,
                             nullptr, nullptr, s, c->launches);
            }
            check_launch("view sobel (batch)");
        }
        LFRV_CUDA(cudaEventRecord(c->vg_ready, s));
    }
    for (size_t q = 0; q < batched.size(); ++q) {
        const Slot &sl = batched[q];
        const lfrv_view_job &J = jobs[sl.job];
        lfrv_ctx *l = c->lanes[q % kLanes];
        const Geometry &G = sl.G;
        Workspace &lw = l->ws;
        lw.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
        // no dtau/dz: IBR_gradient's weights multiply it by the gradient of U = 0 (as in lfrv_render_view_dev)
        // k_tau counts the inverse map's buckets as it writes tau (no separate count pass)
        warp(l, G.V, G.w, G.h, J.d_depth, J.cams, J.target, nullptr, nullptr, lw.tau.as<float>(), nullptr, nullptr,
             nullptr, &G);
        float *U = base + sl.off;
        // the shared view gradients are written (and so the views are uploaded, which the context stream waited for)
        LFRV_CUDA(cudaStreamWaitEvent(l->stream, c->vg_ready, 0));
        gradient_prepare(l, *J.cfg, G, J.d_views, lw.tau.as<float>(), nullptr, nullptr, U, U + 3 * G.N, U + 4 * G.N,
                         sl.seeded ? U + 17 * G.N + 16 : nullptr, nullptr, ws.vg_pool.as<char>() + vg_off[q]);
        // keep this job's hole-fill iteration count (state slot 8) beside its CG state
        double *st = reinterpret_cast<double *>(U + 14 * G.N);
        LFRV_CUDA(cudaMemcpyAsync(st + 6, lw.state.as<double>() + 8, sizeof(double), cudaMemcpyDeviceToDevice,
                                  l->stream));
    }
    for (int k = 0; k < kLanes; ++k) {
        LFRV_CUDA(cudaEventRecord(c->lane_done[k], c->lanes[k]->stream));
        LFRV_CUDA(cudaStreamWaitEvent(s, c->lane_done[k], 0));
    }
    if (views_ready) LFRV_CUDA(cudaStreamWaitEvent(s, views_ready, 0));
    // the other jobs, one after another on the context stream
    for (int j = 0; j < count; ++j) {
        const lfrv_view_job &J = jobs[j];
        const Geometry G = geometry(*J.cfg);
        bool is_batched = false;
        for (const Slot &b : batched) is_batched = is_batched || b.job == j;
        for (int t : tv_idx) is_batched = is_batched || t == j;
        if (is_batched) continue;
        ws.tau.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
        ws.dp.ensure(sizeof(float) * 2 * (size_t)G.V * G.n);
        warp(c, G.V, G.w, G.h, J.d_depth, J.cams, J.target, nullptr, nullptr, ws.tau.as<float>(), ws.dp.as<float>(),
             nullptr);
        {
            // a job outside the batched CG: report what is pending first, then run it to the end and collect its
            // statistics and barrier status before the next job reuses the state slots
            sync(c);
            finish_stats(c);
            if (J.algorithm == 0)
                color_solve(c, *J.cfg, J.d_views, ws.tau.as<float>(), ws.dp.as<float>(), nullptr, J.d_out, J.stats);
            else
                gradient_solve(c, *J.cfg, J.d_views, ws.tau.as<float>(), ws.dp.as<float>(), nullptr, J.d_out, J.stats);
            sync(c);
            finish_stats(c);
        }
    }
    // seeds of the warm-started jobs: the network, one target after another on the context stream
    for (const Slot &sl : batched)
        if (sl.seeded) {
            float *U = base + sl.off;
            warmstart_predict_async(net, sl.G.H, sl.G.W, U + 17 * sl.G.N + 16, U, U + 14 * sl.G.N + 16);
        }
    // energy traces of the batched jobs: one region of ws.trace per job that asks for one
    std::vector<size_t> trace_off(batched.size(), 0);
    size_t trace_total = 0;
    for (size_t q = 0; q < batched.size(); ++q) {
        const lfrv_stats *st = jobs[batched[q].job].stats;
        trace_off[q] = trace_total;
        if (st && st->energy_trace && st->trace_capacity > 0) trace_total += (size_t)st->trace_capacity;
    }
    if (trace_total) ws.trace.ensure(sizeof(double) * trace_total);
    // A job with at least as many 64 x 16 tiles as the batched launch has resident blocks fills the GPU on its own:
    // it gains nothing from sharing a launch, so it runs the single-target persistent CG (shared-memory resident
    // or TMA form) on its pool buffers, one after another on the context stream. The others share k_cg_batch.
    const int resident = cg_batch_resident_blocks();
    // a job's final output (the CG's iterate) to its host destination, after what the context stream has queued
    auto send = [&](const Slot &sl) {
        if (!host_out || !host_out[sl.job] || !sent) return;
        cudaStream_t cs = copy_stream(c);
        LFRV_CUDA(cudaEventRecord(c->out_ready, s));
        LFRV_CUDA(cudaStreamWaitEvent(cs, c->out_ready, 0));
        LFRV_CUDA(cudaMemcpyAsync(host_out[sl.job], base + sl.off + (sl.seeded ? 14 * sl.G.N + 16 : 0),
                                  sizeof(float) * 3 * sl.G.N, cudaMemcpyDeviceToHost, cs));
        sent[sl.job] = 1;
    };
    std::vector<size_t> grouped;
    for (size_t q = 0; q < batched.size(); ++q) {
        const Slot &sl = batched[q];
        const long long ntiles = (long long)((sl.G.W + 63) / 64) * ((sl.G.H + 15) / 16);
        if (ntiles < resident) {
            grouped.push_back(q);
            continue;
        }
        const lfrv_config &cfg = *jobs[sl.job].cfg;
        const lfrv_stats *jst = jobs[sl.job].stats;
        const bool traced = jst && jst->energy_trace && jst->trace_capacity > 0;
        float *U = base + sl.off;
        const size_t N = sl.G.N;
        const size_t np = (size_t)persistent_partials();
        double *part = partial_buf(c, 8 * np);
        const GridBarrier gb = fresh_barrier(c);
        LFRV_CUDA(launch_cg_persistent(sl.G.W, sl.G.H, U + 3 * N, U + 4 * N, sl.seeded ? U + 14 * N + 16 : U,
                                       U + 5 * N, U + 8 * N, U + 11 * N, part, part + 4 * np, gb, cfg.cg_max_iter,
                                       cfg.cg_gap_tol, reinterpret_cast<double *>(U + 14 * N), s, c->launches,
                                       sl.seeded ? U : nullptr, traced ? ws.trace.as<double>() + trace_off[q] : nullptr,
                                       traced ? jst->trace_capacity : 0));
        check_launch("batched job CG");
        send(sl);
    }
    // the CG of the other gradient jobs, in launches of at most `resident` jobs
    for (size_t first = 0; first < grouped.size(); first += (size_t)resident) {
        const size_t cnt = std::min(grouped.size() - first, (size_t)resident);
        std::vector<CgProblem> probs(cnt);
        std::vector<int> tiles(cnt);
        long long total = 0;
        for (size_t q = 0; q < cnt; ++q) {
            const Geometry &G = batched[grouped[first + q]].G;
            tiles[q] = ((G.W + 63) / 64) * ((G.H + 15) / 16);
            total += tiles[q];
        }
        // blocks in proportion to the tiles, at least one each, no more than resident in all
        std::vector<int> nb(cnt);
        int used = 0;
        for (size_t q = 0; q < cnt; ++q) {
            nb[q] = std::max(1, (int)((long long)resident * tiles[q] / std::max(1LL, total)));
            nb[q] = std::min(nb[q], tiles[q]);
            used += nb[q];
        }
        while (used > resident) {  // trim the largest allocations
            size_t big = 0;
            for (size_t q = 1; q < cnt; ++q)
                if (nb[q] > nb[big]) big = q;
            --nb[big];
            --used;
        }
        std::vector<int> block_prob(used);
        int b0 = 0;
        for (size_t q = 0; q < cnt; ++q) {
            const Slot &sl = batched[grouped[first + q]];
            const lfrv_config &cfg = *jobs[sl.job].cfg;
            float *U = base + sl.off;
            CgProblem &P = probs[q];
            P.W = sl.G.W;
            P.H = sl.G.H;
            P.tiles_x = (sl.G.W + 63) / 64;
            P.ntiles = tiles[q];
            P.b0 = b0;
            P.nb = nb[q];
            P.max_iter = cfg.cg_max_iter;
            P.gap_tol = cfg.cg_gap_tol;
            P.gx = U + 3 * sl.G.N;
            P.gy = U + 4 * sl.G.N;
            P.U = sl.seeded ? U + 14 * sl.G.N + 16 : U;
            P.r = U + 5 * sl.G.N;
            P.dA = U + 8 * sl.G.N;
            P.dB = U + 11 * sl.G.N;
            P.state = reinterpret_cast<double *>(U + 14 * sl.G.N);
            P.U0 = sl.seeded ? U : nullptr;
            const lfrv_stats *jst = jobs[sl.job].stats;
            const bool traced = jst && jst->energy_trace && jst->trace_capacity > 0;
            P.trace = traced ? ws.trace.as<double>() + trace_off[grouped[first + q]] : nullptr;
            P.trace_cap = traced ? jst->trace_capacity : 0;
            for (int k = 0; k < nb[q]; ++k) block_prob[b0 + k] = (int)q;
            b0 += nb[q];
        }
        ws.batch_meta.ensure(sizeof(CgProblem) * cnt + sizeof(int) * (used + cnt) + 64);
        char *meta = ws.batch_meta.as<char>();
        CgProblem *d_probs = reinterpret_cast<CgProblem *>(meta);
        int *d_block_prob = reinterpret_cast<int *>(meta + sizeof(CgProblem) * cnt);
        int *d_done = d_block_prob + used;
        LFRV_CUDA(cudaMemcpyAsync(d_probs, probs.data(), sizeof(CgProblem) * cnt, cudaMemcpyHostToDevice, s));
        LFRV_CUDA(cudaMemcpyAsync(d_block_prob, block_prob.data(), sizeof(int) * used, cudaMemcpyHostToDevice, s));
        double *part = partial_buf(c, (size_t)8 * used);
        const GridBarrier gb = fresh_barrier(c);
        LFRV_CUDA(launch_cg_batch(d_probs, d_block_prob, (int)cnt, used, part, part + 4 * (size_t)used, d_done, gb, s,
                                  c->launches));
        for (size_t q = 0; q < cnt; ++q) send(batched[grouped[first + q]]);
        // the next launch rewrites the descriptors in batch_meta (the host vectors were staged by the copies)
        if (first + cnt < grouped.size()) LFRV_CUDA(cudaStreamSynchronize(s));
    }
    // the corrected IBR_color jobs in lockstep (beside the batched CG on the context stream): every round enqueues
    // each running job's certificate, waits once for all of them, then enqueues each job's next FISTA step
    {
        std::vector<size_t> running;
        for (size_t q = 0; q < tv.size(); ++q) running.push_back(q);
        while (!running.empty()) {
            for (size_t q : running) tv[q].eval();
            for (size_t q : running) LFRV_CUDA(cudaStreamSynchronize(c->tv_jobs[q]->stream));
            std::vector<size_t> next;
            for (size_t q : running) {
                TvSolve &ts = tv[q];
                if (!ts.decide()) {
                    ts.step();
                    next.push_back(q);
                    continue;
                }
                ts.finish();
                const lfrv_view_job &J = jobs[tv_idx[q]];
                lfrv_ctx *l = c->tv_jobs[q];
                LFRV_CUDA(cudaMemcpyAsync(J.d_out, l->ws.U.p, sizeof(float) * 3 * ts.G.N, cudaMemcpyDeviceToDevice,
                                          l->stream));
                if (J.stats) {
                    J.stats->outer_iterations = ts.k;
                    J.stats->meta_iterations = 1;
                    J.stats->stop_reason = (J.cfg->cg_gap_tol > 0 && ts.gap <= J.cfg->cg_gap_tol) ? 4 : 0;
                    J.stats->energy = ts.E;
                    J.stats->gap = ts.gap;
                    J.stats->trace_length = ts.st ? ts.trace_pos : 0;
                }
            }
            running.swap(next);
        }
        for (lfrv_ctx *l : c->tv_jobs) {
            LFRV_CUDA(cudaStreamSynchronize(l->stream));
            c->launches.add((int)l->launches.n);
            l->launches.n = 0;
            finish_stats(l);  // barrier status of the FGP launches
        }
    }
    for (const Slot &sl : batched)
        if (!(sent && sent[sl.job]))
            LFRV_CUDA(cudaMemcpyAsync(jobs[sl.job].d_out, base + sl.off + (sl.seeded ? 14 * sl.G.N + 16 : 0),
                                      sizeof(float) * 3 * sl.G.N, cudaMemcpyDeviceToDevice, s));
    sync(c);
    for (lfrv_ctx *l : c->lanes) {
        c->launches.add((int)l->launches.n);
        finish_stats(l);  // the lanes' barrier status (hole filling)
    }
    for (const Slot &sl : batched) {
        lfrv_stats *st = jobs[sl.job].stats;
        if (!st) continue;
        double state[8];
        LFRV_CUDA(cudaMemcpy(state, base + sl.off + 14 * sl.G.N, sizeof(state), cudaMemcpyDeviceToHost));
        st->outer_iterations = (int)state[5];
        st->gap = state[4];
        st->energy = state[3];
        st->hole_fill_iterations = (int)state[6];
        st->stop_reason = (jobs[sl.job].cfg->cg_gap_tol > 0 && state[4] <= jobs[sl.job].cfg->cg_gap_tol) ? 4 : 0;
        if (st->energy_trace && st->trace_capacity > 0) {
            const size_t q = (size_t)(&sl - batched.data());
            st->trace_length = std::min(st->outer_iterations, st->trace_capacity);
            if (st->trace_length > 0)
                LFRV_CUDA(cudaMemcpy(st->energy_trace, ws.trace.as<double>() + trace_off[q],
                                     sizeof(double) * st->trace_length, cudaMemcpyDeviceToHost));
        }
    }
    finish_stats(c);
}

extern "C" int lfrv_render_views_dev(lfrv_ctx *ctx, const lfrv_view_job *jobs, int count) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    render_views(ctx, jobs, count);
    LFRV_API_END
}

extern "C" int lfrv_render_views_warm_dev(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_view_job *jobs,
                                          int count) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!net) return fail(LFRV_E_ARG, "null network");
    render_views(ctx, jobs, count, net);
    warmstart_check(net);
    LFRV_API_END
}

// Host-buffer batched targets: the jobs' views, depth maps and outputs are host pointers. Each distinct input
// buffer (same pointer and size, as when many targets share one light field) is uploaded once into one device
// pool: the depth maps on the context stream (the warp stage reads them first), the colour views on the copy stream
// while the warp stage runs. The batch runs as lfrv_render_views_dev would. An IBR_gradient job whose output is
// pinned host memory is downloaded on the copy stream as soon as its CG is done, while the next jobs run; the other
// outputs are copied back at the end. The call returns once every output is in host memory.
static void render_views_host(lfrv_ctx *c, const lfrv_view_job *jobs, int count, lfrv_warmstart *net) {
    if (count <= 0 || !jobs) raise(LFRV_E_ARG, "empty batch");
    struct Input {
        const void *host;
        size_t bytes, off;
        bool depth;  // some job's depth maps: needed by the warp stage
    };
    std::vector<Input> inputs;
    auto place = [&](const void *p, size_t bytes, bool depth) -> size_t {
        for (Input &in : inputs)
            if (in.host == p && in.bytes == bytes) {
                in.depth = in.depth || depth;
                return in.off;
            }
        const size_t off = inputs.empty() ? 0 : (inputs.back().off + inputs.back().bytes + 255) / 256 * 256;
        inputs.push_back({p, bytes, off, depth});
        return off;
    };
    std::vector<size_t> off_views(count), off_depth(count), off_out(count);
    size_t out_bytes = 0;
    for (int j = 0; j < count; ++j) {
        const lfrv_view_job &J = jobs[j];
        if (!J.cfg || !J.d_views || !J.d_depth || !J.d_out) raise(LFRV_E_ARG, "job %d: null argument", j);
        const Geometry G = geometry(*J.cfg);
        const size_t vb = (size_t)G.V * 3 * G.n * (J.cfg->bf16_storage ? 2 : 4);
        off_views[j] = place(J.d_views, vb, false);
        off_depth[j] = place(J.d_depth, (size_t)G.V * 3 * G.n * sizeof(float), true);
        off_out[j] = out_bytes;
        out_bytes += (3 * G.N * sizeof(float) + 255) / 256 * 256;
    }
    const size_t in_bytes = inputs.back().off + inputs.back().bytes;
    c->ws.hb_in.ensure(in_bytes);
    c->ws.hb_out.ensure(out_bytes);
    char *din = c->ws.hb_in.as<char>(), *dout = c->ws.hb_out.as<char>();
    cudaStream_t cs = copy_stream(c);
    // the copy stream starts after what the context stream has queued (an earlier call may still read the pool)
    LFRV_CUDA(cudaEventRecord(c->up_start, c->stream));
    LFRV_CUDA(cudaStreamWaitEvent(cs, c->up_start, 0));
    for (const Input &in : inputs)
        LFRV_CUDA(cudaMemcpyAsync(din + in.off, in.host, in.bytes, cudaMemcpyHostToDevice, in.depth ? c->stream : cs));
    LFRV_CUDA(cudaEventRecord(c->up_views, cs));
    // pinned destinations take the early download; a pageable one would make each copy wait on the host
    std::vector<float *> host_out(count, nullptr);
    for (int j = 0; j < count; ++j) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, jobs[j].d_out) == cudaSuccess && a.type == cudaMemoryTypeHost)
            host_out[j] = jobs[j].d_out;
        else
            cudaGetLastError();
    }
    std::vector<char> sent(count, 0);
    std::vector<lfrv_view_job> dj(jobs, jobs + count);
    for (int j = 0; j < count; ++j) {
        dj[j].d_views = reinterpret_cast<const float *>(din + off_views[j]);
        dj[j].d_depth = reinterpret_cast<const float *>(din + off_depth[j]);
        dj[j].d_out = reinterpret_cast<float *>(dout + off_out[j]);
    }
    try {
        render_views(c, dj.data(), count, net, host_out.data(), sent.data(), c->up_views);
    } catch (...) {
        cudaStreamSynchronize(cs);  // no copy into the caller's buffers outlives the call
        throw;
    }
    for (int j = 0; j < count; ++j) {
        if (sent[j]) continue;
        const Geometry G = geometry(*jobs[j].cfg);
        LFRV_CUDA(cudaMemcpyAsync(jobs[j].d_out, dout + off_out[j], 3 * G.N * sizeof(float), cudaMemcpyDeviceToHost,
                                  c->stream));
    }
    sync(c);
    LFRV_CUDA(cudaStreamSynchronize(cs));
}

extern "C" int lfrv_render_views(lfrv_ctx *ctx, const lfrv_view_job *jobs, int count) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    render_views_host(ctx, jobs, count, nullptr);
    LFRV_API_END
}

extern "C" int lfrv_render_views_warm(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_view_job *jobs, int count) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!net) return fail(LFRV_E_ARG, "null network");
    render_views_host(ctx, jobs, count, net);
    warmstart_check(net);
    LFRV_API_END
}

// ------------------------------------------------------------------ IBR_video
// TargetView::move (sources/openGL/view.cpp:1744-1759), in its float arithmetic: the centre moves from camera a's
// towards camera b's by frame / 1000 of the way, the rotation is camera a's turned about the y axis by frame * 0.0003
// rad, K and the size stay the target's.
extern "C" int lfrv_video_camera(const lfrv_camera *a, const lfrv_camera *b, const lfrv_camera *target, int frame,
                                 lfrv_camera *out) {
    if (!a || !b || !target || !out || frame < 0) return fail(LFRV_E_ARG, "bad arguments");
    float Ca[3], Cb[3];
    for (int i = 0; i < 3; ++i) {  // C = -R^T t
        Ca[i] = -(a->R[0 * 3 + i] * a->t[0] + a->R[1 * 3 + i] * a->t[1] + a->R[2 * 3 + i] * a->t[2]);
        Cb[i] = -(b->R[0 * 3 + i] * b->t[0] + b->R[1 * 3 + i] * b->t[1] + b->R[2 * 3 + i] * b->t[2]);
    }
    const float step = 1000.0f, angle = 0.0003f;
    const float count = (float)frame;
    float C[3];
    for (int i = 0; i < 3; ++i) C[i] = Ca[i] + count * (Cb[i] - Ca[i]) / step;
    const float cs = std::cos(count * angle), sn = std::sin(count * angle);
    const float Ry[9] = {cs, 0.0f, sn, 0.0f, 1.0f, 0.0f, -sn, 0.0f, cs};
    lfrv_camera o = *target;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            o.R[r * 3 + c] = Ry[r * 3 + 0] * a->R[0 * 3 + c] + Ry[r * 3 + 1] * a->R[1 * 3 + c] + Ry[r * 3 + 2] * a->R[2 * 3 + c];
    for (int r = 0; r < 3; ++r) o.t[r] = -(o.R[r * 3 + 0] * C[0] + o.R[r * 3 + 1] * C[1] + o.R[r * 3 + 2] * C[2]);
    *out = o;
    return LFRV_OK;
}

// The IBR_video loop (sources/main.cpp:359-403) over one static light field: frames first_frame .. first_frame +
// nframes - 1, each a target camera moved by lfrv_video_camera from views cam_a and cam_b, all rendered as one batch.
extern "C" int lfrv_render_video_dev(lfrv_ctx *ctx, const lfrv_config *cfg, int algorithm, const float *d_views,
                                     const float *d_depth, const lfrv_camera *cams, int cam_a, int cam_b,
                                     const lfrv_camera *target, int first_frame, int nframes, float *d_out,
                                     lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!cfg || !d_views || !d_depth || !cams || !target || !d_out || nframes < 1 || first_frame < 0)
        return fail(LFRV_E_ARG, "bad arguments");
    if (cam_a < 0 || cam_a >= cfg->nviews || cam_b < 0 || cam_b >= cfg->nviews)
        return fail(LFRV_E_ARG, "camera indices %d, %d outside the %d views", cam_a, cam_b, cfg->nviews);
    const Geometry G = geometry(*cfg);
    std::vector<lfrv_camera> tcams(nframes);
    std::vector<lfrv_view_job> jobs(nframes);
    for (int f = 0; f < nframes; ++f) {
        const int rc = lfrv_video_camera(&cams[cam_a], &cams[cam_b], target, first_frame + f, &tcams[f]);
        if (rc != LFRV_OK) return rc;
        jobs[f] = lfrv_view_job{cfg, algorithm, d_views, d_depth, cams, &tcams[f], d_out + (size_t)f * 3 * G.N,
                                stats ? &stats[f] : nullptr};
    }
    render_views(ctx, jobs.data(), nframes);
    LFRV_API_END
}

static cudaStream_t copy_stream(lfrv_ctx *c) {
    if (!c->copy_stream) {
        LFRV_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        LFRV_CUDA(cudaEventCreateWithFlags(&c->up_start, cudaEventDisableTiming));
        LFRV_CUDA(cudaEventCreateWithFlags(&c->up_views, cudaEventDisableTiming));
        LFRV_CUDA(cudaEventCreateWithFlags(&c->out_ready, cudaEventDisableTiming));
        for (auto &e : c->up_depth) LFRV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    return c->copy_stream;
}

extern "C" int lfrv_render_view(lfrv_ctx *ctx, const lfrv_config *cfg, int algorithm, const float *views,
                                const float *depth, const lfrv_camera *cams, const lfrv_camera *target, float *out,
                                lfrv_stats *stats) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (!cfg || !views || !depth || !out || !cams || !target) return fail(LFRV_E_ARG, "null argument");
    if (cfg->bf16_storage) return fail(LFRV_E_ARG, "bf16_storage needs device views (the *_dev entry points)");
    const Geometry G = geometry(*cfg);
    if (G.V < 1 || G.V > kMaxViews) return fail(LFRV_E_ARG, "bad view count");
    const size_t n = G.n, V = G.V, per_view = 3 * n * sizeof(float);
    Workspace &ws = ctx->ws;
    ws.in_views.ensure(V * per_view);
    ws.depth.ensure(V * per_view);
    ws.out_img.ensure(sizeof(float) * 3 * G.N);
    // uploads on the copy stream, after whatever the context stream has queued on these buffers; the depth
    // maps first, in up to 4 chunks of views, then the colour views
    cudaStream_t cs = copy_stream(ctx);
    UploadPlan plan;
    auto upload = [&] {
        LFRV_CUDA(cudaEventRecord(ctx->up_start, ctx->stream));
        LFRV_CUDA(cudaStreamWaitEvent(cs, ctx->up_start, 0));
        plan.chunks = G.V < 4 ? G.V : 4;
        int v0 = 0;
        for (int k = 0; k < plan.chunks; ++k) {
            const int v1 = (int)((V * (size_t)(k + 1)) / plan.chunks);
            LFRV_CUDA(cudaMemcpyAsync(ws.depth.as<char>() + v0 * per_view,
                                      reinterpret_cast<const char *>(depth) + v0 * per_view,
                                      (size_t)(v1 - v0) * per_view, cudaMemcpyHostToDevice, cs));
            LFRV_CUDA(cudaEventRecord(ctx->up_depth[k], cs));
            plan.v_end[k] = v1;
            plan.depth_ready[k] = ctx->up_depth[k];
            v0 = v1;
        }
        LFRV_CUDA(cudaMemcpyAsync(ws.in_views.p, views, V * per_view, cudaMemcpyHostToDevice, cs));
        LFRV_CUDA(cudaEventRecord(ctx->up_views, cs));
        plan.views_ready = ctx->up_views;
    };
    // a repeated call (same host buffers and arguments) replays its captured graph: uploads, warp, solve and
    // the download in one launch
    const bool replayed =
        graph_eligible(ctx, *cfg, algorithm, target, stats) &&
        render_graph(ctx, render_key(ctx, *cfg, algorithm, views, depth, out, cams, target), stats, [&] {
            upload();
            render_view_body(ctx, *cfg, algorithm, ws.in_views.as<float>(), ws.depth.as<float>(), cams, target,
                             ws.out_img.as<float>(), nullptr, &plan, out);
        });
    if (!replayed) {
        upload();
        render_view_impl(ctx, *cfg, algorithm, ws.in_views.as<float>(), ws.depth.as<float>(), cams, target,
                         ws.out_img.as<float>(), stats, &plan, out);
    }
    LFRV_API_END
}

// ====================================================================== stage calls
namespace {

struct StageInputs {
    Geometry G;
    const float *img = nullptr, *tau2 = nullptr, *dp2 = nullptr;
};

StageInputs stage_inputs(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                         const float *dpart) {
    StageInputs si;
    si.G = geometry(*cfg);
    HostIO io{ctx};
    const size_t n = si.G.n, V = si.G.V;
    std::vector<float> zeros;
    if (!views) {
        zeros.assign(V * 3 * n, 0.0f);
        views = zeros.data();
    }
    si.img = io.up(ctx->ws.in_views, views, V * 3 * n);
    const float *dt = io.up(ctx->ws.in_tau, tau, V * (size_t)tau_ch * n);
    const float *dd = io.up(ctx->ws.in_dpart, dpart, V * 3 * n);
    prepare_geometry_inputs(ctx, si.G, dt, tau_ch, dd);
    si.tau2 = ctx->ws.tau.as<float>();
    si.dp2 = ctx->ws.dp.as<float>();
    sync(ctx);
    return si;
}

}  // namespace

extern "C" int lfrv_stage_visibility(lfrv_ctx *ctx, const lfrv_config *cfg, const float *tau, int tau_channels,
                                     float *coverage, uint8_t *vis) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, nullptr, tau, tau_channels, nullptr);
    const Buckets B = build_buckets(ctx, si.G, si.tau2);
    ColorBuffers b = color_buffers(ctx, si.G);
    launch_coverage(si.G, B, si.tau2, b.cov, b.vis, ctx->stream, ctx->launches);
    check_launch("coverage");
    HostIO io{ctx};
    io.down(coverage, b.cov, si.G.N);
    io.down(vis, b.vis, si.G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_weights(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                                  int tau_channels, const float *dpart, const float *U, const uint8_t *vis, float *gx,
                                  float *gy, float *weights) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, views, tau, tau_channels, dpart);
    const Geometry &G = si.G;
    ColorBuffers b = color_buffers(ctx, G);
    HostIO io{ctx};
    io.up(ctx->ws.U, U, 3 * G.N);
    io.up(ctx->ws.vis, vis, G.N);
    io.up(ctx->ws.gx, gx, G.N);
    io.up(ctx->ws.gy, gy, G.N);
    launch_sobel(G.W, G.H, 1, ctx->ws.U.as<float>(), 0, G.N, b.gx, b.gy, 0, b.vis, nullptr, ctx->stream,
                 ctx->launches);
    launch_weights(G, b.gx, b.gy, si.tau2, si.dp2, cfg->sigma_sensor, cfg->ugrad_threshold, b.wgt, ctx->stream,
                   ctx->launches);
    check_launch("weights");
    io.down(gx, b.gx, G.N);
    io.down(gy, b.gy, G.N);
    io.down(weights, b.wgt, (size_t)G.V * G.n);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_dataterm(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                                   int tau_channels, const float *weights, const float *U, float *Gout, float *F) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, views, tau, tau_channels, nullptr);
    const Geometry &G = si.G;
    const Buckets B = build_buckets(ctx, G, si.tau2);
    ColorBuffers b = color_buffers(ctx, G);
    HostIO io{ctx};
    io.up(ctx->ws.wgt, weights, (size_t)G.V * G.n);
    io.up(ctx->ws.U, U, 3 * G.N);
    ctx->ws.G.ensure(sizeof(float) * 3 * G.N);
    const float s2 = cfg->sigma_sensor * cfg->sigma_sensor;
    residual(ctx, G, ctx->ws.U.as<float>(), si.img, si.tau2, b.wgt, s2, b.res, 0);
    const float L = (float)(1.0 / cfg->lambda);
    const float fscale = (float)(-1.0 / (double)(cfg->lambda * L));
    const GradientTermBuffers gtb = gradient_term_buffers(ctx, *cfg, G, si.img);
    const GradTerm gt = gradient_residuals(ctx, *cfg, G, gtb, ctx->ws.U.as<float>(), si.img, si.tau2, b.wgt);
    launch_dataterm_F(G, B, si.tau2, b.res, s2, cfg->dt_alpha, fscale, ctx->ws.U.as<float>(), b.F,
                      ctx->ws.G.as<float>(), gt, ctx->stream, ctx->launches);
    check_launch("data term");
    io.down(Gout, ctx->ws.G.as<float>(), 3 * G.N);
    io.down(F, b.F, 3 * G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_rof(lfrv_ctx *ctx, int W, int H, int niter, float tau, float sigma, float lambda,
                              const float *F, const float *g, float *U, float *P) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (W <= 0 || H <= 0 || niter < 0 || !F || !g || !U || !P) return fail(LFRV_E_ARG, "bad arguments");
    const size_t N = (size_t)W * H;
    Workspace &ws = ctx->ws;
    HostIO io{ctx};
    io.up(ws.F, F, 3 * N);
    io.up(ws.g, g, N);
    io.up(ws.U, U, 3 * N);
    io.up(ws.P, P, 6 * N);
    ws.Ua.ensure(3 * N * sizeof(float));
    ws.Pa.ensure(6 * N * sizeof(float));
    ctx->pending = Pending{};
    const int rv = rof_autotune(ctx, W, H, tau, sigma, lambda, ws.U.as<float>(), ws.P.as<float>(), ws.F.as<float>(),
                                ws.g.as<float>());
    const GridBarrier gb = fresh_barrier(ctx);
    LFRV_CUDA(launch_rof_persistent(W, H, niter, tau, sigma, lambda, ws.U.as<float>(), ws.P.as<float>(),
                                    ws.Ua.as<float>(), ws.Pa.as<float>(), ws.F.as<float>(), ws.g.as<float>(), gb, rv,
                                    ctx->stream, ctx->launches));
    const bool odd = (rof_persistent_steps(niter, rv) & 1) != 0;
    io.down(U, odd ? ws.Ua.as<float>() : ws.U.as<float>(), 3 * N);
    io.down(P, odd ? ws.Pa.as<float>() : ws.P.as<float>(), 6 * N);
    sync(ctx);
    finish_stats(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_energy(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                                 int tau_channels, const float *weights, const float *U, const uint8_t *vis,
                                 double *energy, double *e_tv, double *e_data) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, views, tau, tau_channels, nullptr);
    const Geometry &G = si.G;
    ColorBuffers b = color_buffers(ctx, G);
    HostIO io{ctx};
    io.up(ctx->ws.wgt, weights, (size_t)G.V * G.n);
    io.up(ctx->ws.U, U, 3 * G.N);
    io.up(ctx->ws.vis, vis, G.N);
    LFRV_CUDA(cudaMemsetAsync(b.Xq, 0, 2 * G.N * sizeof(float), ctx->stream));
    const float s2 = cfg->sigma_sensor * cfg->sigma_sensor;
    sobel_target(ctx, G, ctx->ws.U.as<float>(), b.Xq, b.Xq + G.N, b.vis, 0);
    residual(ctx, G, ctx->ws.U.as<float>(), si.img, si.tau2, b.wgt, s2, b.res, 1);
    const GradientTermBuffers gtb = gradient_term_buffers(ctx, *cfg, G, si.img);
    if (gtb.on) energy_gradients(ctx, *cfg, G, gtb, ctx->ws.U.as<float>(), si.tau2, b.wgt, 3);
    double sums[4] = {0, 0, 0, 0};
    read_sums(ctx, sums, gtb.on ? 4 : 2);
    if (e_tv) *e_tv = sums[0];
    if (e_data) *e_data = sums[1];
    if (energy)
        *energy = (double)cfg->lambda * sums[0] + (double)cfg->dt_alpha * sums[1] + (double)cfg->dt_beta * sums[3];
    LFRV_API_END
}

extern "C" int lfrv_stage_regularizer(lfrv_ctx *ctx, const lfrv_config *cfg, const float *tau, int tau_channels,
                                      const float *weights, const float *norm_in, float *norm_out, float *g) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, nullptr, tau, tau_channels, nullptr);
    const Geometry &G = si.G;
    const Buckets B = build_buckets(ctx, G, si.tau2);
    ColorBuffers b = color_buffers(ctx, G);
    HostIO io{ctx};
    io.up(ctx->ws.wgt, weights, (size_t)G.V * G.n);
    const float *prior = norm_in ? io.up(ctx->ws.norm, norm_in, G.N) : nullptr;
    const float s2 = cfg->sigma_sensor * cfg->sigma_sensor;
    launch_regweight(G, B, si.tau2, b.wgt, prior, s2, cfg->lambda_max_factor * cfg->lambda, cfg->lambda, (float)G.V,
                     b.g0, b.norm, ctx->stream, ctx->launches);
    launch_blur(G.W, G.H, b.g0, b.tmp, b.g, ctx->stream, ctx->launches);
    check_launch("regularizer");
    io.down(norm_out, b.norm, G.N);
    io.down(g, b.g, G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_initial_image(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                                        int tau_channels, const float *weights, float *U, float *norm) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, views, tau, tau_channels, nullptr);
    const Geometry &G = si.G;
    const Buckets B = build_buckets(ctx, G, si.tau2);
    ColorBuffers b = color_buffers(ctx, G);
    HostIO io{ctx};
    io.up(ctx->ws.wgt, weights, (size_t)G.V * G.n);
    launch_initial_image(G, B, si.tau2, si.img, b.wgt, ctx->ws.U.as<float>(), b.norm, ctx->stream, ctx->launches);
    check_launch("initial image");
    io.down(U, ctx->ws.U.as<float>(), 3 * G.N);
    io.down(norm, b.norm, G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_push_pull(lfrv_ctx *ctx, int W, int H, int faithful, const uint8_t *vis, float *U) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (W <= 0 || H <= 0 || !vis || !U) return fail(LFRV_E_ARG, "bad arguments");
    const size_t N = (size_t)W * H;
    Workspace &ws = ctx->ws;
    HostIO io{ctx};
    io.up(ws.U, U, 3 * N);
    io.up(ws.vis, vis, N);
    ws.pp_img.ensure(sizeof(float) * 3 * (N / 2 + 16));
    ws.pp_vis.ensure(N / 2 + 16 + N);
    ws.pp_tmp.ensure(sizeof(float) * 3 * (N / 2 + (size_t)W + 16));
    ws.pp_orig.ensure(sizeof(float) * 3 * N);
    PushPull pp;
    float *pi = ws.pp_img.as<float>();
    uint8_t *pv = ws.pp_vis.as<uint8_t>();
    pp.vis[0] = pv;
    pv += N;
    for (int l = 1; l <= 10; ++l) {
        const size_t sz = (size_t)(W >> l) * (H >> l);
        pp.img[l] = pi;
        pp.vis[l] = pv;
        pi += 3 * sz;
        pv += sz;
    }
    pp.tmp = ws.pp_tmp.as<float>();
    pp.orig = ws.pp_orig.as<float>();
    launch_push_pull(W, H, faithful != 0, ws.vis.as<uint8_t>(), ws.U.as<float>(), pp, ctx->stream, ctx->launches);
    check_launch("push-pull");
    io.down(U, ws.U.as<float>(), 3 * N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_gradient_visibility(lfrv_ctx *ctx, const lfrv_config *cfg, const float *tau,
                                              int tau_channels, uint8_t *vis) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, nullptr, tau, tau_channels, nullptr);
    const Buckets B = build_buckets(ctx, si.G, si.tau2);
    ColorBuffers b = color_buffers(ctx, si.G);
    launch_vis_any(si.G, B, si.tau2, b.vis, ctx->stream, ctx->launches);
    check_launch("visibility");
    HostIO io{ctx};
    io.down(vis, b.vis, si.G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_hole_fill(lfrv_ctx *ctx, int W, int H, int max_iter, const uint8_t *vis, float *U,
                                    int *iterations) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (W <= 0 || H <= 0 || !vis || !U) return fail(LFRV_E_ARG, "bad arguments");
    const size_t N = (size_t)W * H;
    HostIO io{ctx};
    io.up(ctx->ws.U, U, 3 * N);
    io.up(ctx->ws.vis, vis, N);
    lfrv_stats st;
    std::memset(&st, 0, sizeof(st));
    ctx->pending = Pending{};
    hole_fill_async(ctx, W, H, ctx->ws.vis.as<uint8_t>(), ctx->ws.U.as<float>(), max_iter);
    ctx->pending.stats = &st;
    io.down(U, ctx->ws.U.as<float>(), 3 * N);
    sync(ctx);
    finish_stats(ctx);
    if (iterations) *iterations = st.hole_fill_iterations;
    LFRV_API_END
}

extern "C" int lfrv_stage_u_gradient(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                                     int tau_channels, const float *weights, float *gx, float *gy, float *mask) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    StageInputs si = stage_inputs(ctx, cfg, views, tau, tau_channels, nullptr);
    const Geometry &G = si.G;
    const Buckets B = build_buckets(ctx, G, si.tau2);
    ColorBuffers b = color_buffers(ctx, G);
    HostIO io{ctx};
    io.up(ctx->ws.wgt, weights, (size_t)G.V * G.n);
    ctx->ws.mask.ensure(sizeof(float) * G.N);
    u_gradient(ctx, G, B, si.img, si.tau2, b.wgt, cfg->sigma_sensor * cfg->sigma_sensor, b.gx, b.gy,
               ctx->ws.mask.as<float>());
    io.down(gx, b.gx, G.N);
    io.down(gy, b.gy, G.N);
    io.down(mask, ctx->ws.mask.as<float>(), G.N);
    sync(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_poisson_jacobi(lfrv_ctx *ctx, int W, int H, int iterations, const float *gx,
                                         const float *gy, const float *mask, float *U) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (W < 1 || H < 1 || iterations < 0 || !gx || !gy || !mask || !U) return fail(LFRV_E_ARG, "bad arguments");
    const size_t N = (size_t)W * H;
    HostIO io{ctx};
    io.up(ctx->ws.gx, gx, N);
    io.up(ctx->ws.gy, gy, N);
    io.up(ctx->ws.mask, mask, N);
    io.up(ctx->ws.U, U, 3 * N);
    ctx->ws.Ua.ensure(sizeof(float) * 3 * N);
    ctx->ws.r.ensure(sizeof(float) * 3 * N);
    ctx->ws.tmp.ensure(sizeof(float) * N);
    ctx->pending = Pending{};
    const GridBarrier gb = fresh_barrier(ctx);
    LFRV_CUDA(launch_poisson_jacobi(W, H, iterations, ctx->ws.gx.as<float>(), ctx->ws.gy.as<float>(),
                                    ctx->ws.mask.as<float>(), ctx->ws.U.as<float>(), ctx->ws.Ua.as<float>(),
                                    ctx->ws.r.as<float>(), ctx->ws.tmp.as<float>(), gb, ctx->stream, ctx->launches));
    io.down(U, ctx->ws.U.as<float>(), 3 * N);
    sync(ctx);
    finish_stats(ctx);
    LFRV_API_END
}

extern "C" int lfrv_stage_cg(lfrv_ctx *ctx, int W, int H, int faithful, int max_iter, double gap_tol, const float *gx,
                             const float *gy, float *U, int *iterations, double *gap) {
    LFRV_API_BEGIN
    CTX_CHECK(ctx);
    if (W < 2 || H < 2 || !gx || !gy || !U) return fail(LFRV_E_ARG, "bad arguments");
    const size_t N = (size_t)W * H;
    HostIO io{ctx};
    io.up(ctx->ws.gx, gx, N);
    io.up(ctx->ws.gy, gy, N);
    io.up(ctx->ws.U, U, 3 * N);
    lfrv_stats st;
    std::memset(&st, 0, sizeof(st));
    ctx->pending = Pending{};
    if (faithful) {
        st.outer_iterations = cg_faithful(ctx, W, H, ctx->ws.gx.as<float>(), ctx->ws.gy.as<float>(),
                                          ctx->ws.U.as<float>());
    } else {
        cg_persistent_async(ctx, W, H, max_iter, gap_tol, ctx->ws.gx.as<float>(), ctx->ws.gy.as<float>(),
                            ctx->ws.U.as<float>());
        ctx->pending.stats = &st;
        ctx->pending.gap_tol = gap_tol;
    }
    io.down(U, ctx->ws.U.as<float>(), 3 * N);
    sync(ctx);
    finish_stats(ctx);
    if (iterations) *iterations = st.outer_iterations;
    if (gap) *gap = st.gap;
    LFRV_API_END
}
