// kernels.h -- host-side declarations of the lfrv kernel launchers (internal to liblfrv).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace lfrv {

struct KernelProfiler;

// Counts kernel launches issued by a context; optionally times them per kernel name.
struct LaunchCounter {
    long long n = 0;
    KernelProfiler *prof = nullptr;
    void add(int k) { n += k; }
};

// Records a CUDA event pair on `st` around its scope when the context profiles (no host synchronisation).
struct ProfScope {
    ProfScope(LaunchCounter &lc, const char *name, cudaStream_t st);
    ~ProfScope();
    KernelProfiler *p;
    int slot;
    cudaStream_t st;
};

// Sizes of one solve: V views of w x h source pixels, target W x H = (dsf w) x (dsf h).
struct Geometry {
    int V, w, h, n, W, H, dsf;
    size_t N;
};

// Inverse footprint map: source pixels of all views bucketed by footprint anchor.
struct Buckets {
    int BW, BH, nb;                     // bucket grid (W + ks - 1) x (H + ks - 1)
    unsigned int *count, *start;        // nb, nb + 1
    unsigned int *entries;              // V * n capacity, (view << 24) | pixel
    unsigned long long *mask;           // mask_words x nb: bit v % 64 of word v / 64 set when view v lands in the
                                        // bucket (word-major: word w of bucket b at mask[w * nb + b])
    int mask_words;                     // ceil(V / 64)
    unsigned int *block_sums, *block_offsets, *block_sums2, *block_offsets2, *total, *total2;
};

// ---- warp stage (kernels_warp.cu)
// Per input view, the cameras folded by the host: x_h = M (z (x, y, 1)) + b with M = K_u R_u R_k^T K_k^-1 and
// b = K_u (t_u - R_u R_k^T t_k). Passed by value as a kernel parameter (at most kMaxViews views).
constexpr int kMaxViews = 255;
struct WarpCams {
    float M[kMaxViews][9];
    float b[kMaxViews][3];
};
// Cameras of the warps-from-depth path (views 0..V-1, then the target at V): fx, fy, cx, cy, R (9, row-major),
// C (3), P = K [R | t] (12, row-major).
struct WfdCams {
    float c[kMaxViews + 1][28];
};
void launch_warp_from_depth(int V, int w, int h, int dsf, const float *depth, int depth_channels, const WfdCams &cams,
                            int W, int H, int faithful, unsigned int *ukey, float *tau, cudaStream_t st,
                            LaunchCounter &lc);
// Radial to orthographic depth in place; kinv.M[v] holds K^-1 of view v.
void launch_radial_to_ortho(int V, int w, int h, const WarpCams &kinv, float *depth, cudaStream_t st,
                            LaunchCounter &lc);
void launch_zbuffer_clear(int W, int H, unsigned long long *zkey, cudaStream_t st, LaunchCounter &lc);
// Words of the z-buffer splat's queue of large quads for V views of w x h (launch_zbuffer_splat's defer_q).
size_t zsplat_defer_words(int V, int w, int h);
void launch_zbuffer_splat(int V, int w, int h, const float *depth, const WarpCams &cams, int W, int H,
                          unsigned long long *zkey, unsigned int *defer_q, cudaStream_t st, LaunchCounter &lc);
void launch_zbuffer_resolve(int W, int H, const unsigned long long *zkey, float *zbuf, cudaStream_t st,
                            LaunchCounter &lc);
// tau3/dpart3: reference format (V x 3 x n); tau2/dp2: solver format (V x 2 x n), dp2 premultiplied by sigma_z.
// Any output may be null.
// The inverse map's per-bucket counts (and view masks) that k_tau can accumulate while it writes tau, so the
// bucket build needs no count pass of its own (count and mask zeroed beforehand).
struct BucketCount {
    unsigned int *count = nullptr;
    unsigned long long *mask = nullptr;  // view masks: word w of bucket b at mask[w * nb + b]
    int dsf = 0, BW = 0, nb = 0;
};
void launch_tau(int V, int w, int h, const float *depth, const WarpCams &cams, int W, int H, const float *zbuf,
                float *tau3, float *dpart3, float *tau2, float *dp2, cudaStream_t st, LaunchCounter &lc,
                const BucketCount *bc = nullptr, const unsigned long long *zkey = nullptr);  // zbuf null: read zkey

// ---- solver stage (kernels_solver.cu)
void launch_bucket_build(const Geometry &G, const float *tau, Buckets &B, cudaStream_t st, LaunchCounter &lc,
                         bool counted = false);
void launch_residual(const Geometry &G, const float *U, const float *img, const float *tau, const float *wgt, float s2,
                     float *res, double *partial, cudaStream_t st, LaunchCounter &lc, bool splat_set = false);
int residual_partials(const Geometry &G);
// wgt: FP32, or BF16 with bf16 = true (the BF16 storage mode of IBR_gradient).
void launch_weights(const Geometry &G, const float *gx, const float *gy, const float *tau, const float *dp, float sigma,
                    float thr, void *wgt, cudaStream_t st, LaunchCounter &lc, bool bf16 = false);
void launch_coverage(const Geometry &G, const Buckets &B, const float *tau, float *cov, uint8_t *vis, cudaStream_t st,
                     LaunchCounter &lc);
void launch_vis_any(const Geometry &G, const Buckets &B, const float *tau, uint8_t *vis, cudaStream_t st,
                    LaunchCounter &lc);
void launch_initial_image(const Geometry &G, const Buckets &B, const float *tau, const float *img, const float *wgt,
                          float *U, float *norm, cudaStream_t st, LaunchCounter &lc);
// Learned warm start input (NHWC BF16, kLearnChannels per target pixel) from the IBR_gradient set-up products
// and the first kLearnViews views splatted one at a time.
constexpr int kLearnChannels = 48, kLearnViews = 8;
void launch_learn_input(const Geometry &G, const Buckets &B, const float *tau, const void *img, const void *wgt,
                        const float *U, const float *gx, const float *gy, const uint8_t *vis, void *out,
                        cudaStream_t st, LaunchCounter &lc, bool bf16 = false);
// Gradient data term of the ISTA step (dt_beta > 0): per-view residuals resg (3 x n each) and their weights.
struct GradTerm {
    const float *resg;  // nullptr: no gradient term
    float beta, step;
    int gw;
};
void launch_dataterm_F(const Geometry &G, const Buckets &B, const float *tau, const float *res, float s2, float alpha,
                       float fscale, const float *U, float *F, float *G_out, const GradTerm &gt, cudaStream_t st,
                       LaunchCounter &lc);
void launch_laplacian(int W, int H, int planes, const float *in, float *out, cudaStream_t st, LaunchCounter &lc);
void launch_residual_grad(const Geometry &G, const float *lapU, const float *img, const float *tau, const float *wgt,
                          int gw, float *resg, cudaStream_t st, LaunchCounter &lc);
int energy_grad_partials(const Geometry &G);
void launch_energy_grad(const Geometry &G, const float *ugrad, const float *vgrad, const float *tau, const float *wgt,
                        float s2, int gw, double *partial, cudaStream_t st, LaunchCounter &lc);
void launch_regweight(const Geometry &G, const Buckets &B, const float *tau, const float *wgt, const float *norm_prior,
                      float s2, float lmax, float lmin, float mmax, float *g0, float *norm_out, cudaStream_t st,
                      LaunchCounter &lc);
void launch_u_gradient(const Geometry &G, const Buckets &B, const float *tau, const float *vgrad, const float *wgt,
                       float s2, float *gx, float *gy, float *mask, cudaStream_t st, LaunchCounter &lc);
// img, vgrad, wgt: FP32, or BF16 with bf16 = true; U, gx, gy, mask FP32 either way.
void launch_gradient_setup(const Geometry &G, const Buckets &B, const float *tau, const void *img, const void *vgrad,
                           const void *wgt, float s2, uint8_t *vis, float *U, float *gx, float *gy, float *mask,
                           cudaStream_t st, LaunchCounter &lc, bool bf16 = false);
// Luminance Sobel of BF16 views into BF16 gradients.
void launch_view_sobel_bf16(int W, int H, int count, const void *rgb, size_t in_stride, size_t ch_stride, void *gx,
                            void *gy, size_t out_stride, cudaStream_t st, LaunchCounter &lc);
void launch_sobel(int W, int H, int count, const float *rgb, size_t in_stride, size_t ch_stride, float *gx, float *gy,
                  size_t out_stride, const uint8_t *vis, double *abs_partial, cudaStream_t st, LaunchCounter &lc);
int sobel_partials(int W, int H);
void launch_moving(size_t N, const float *A, const float *B, float thr, double *partial, cudaStream_t st,
                   LaunchCounter &lc);
int moving_partials(size_t N);
void set_gaussian(const float k[11]);
void launch_blur(int W, int H, const float *in, float *tmp, float *out, cudaStream_t st, LaunchCounter &lc);
void launch_reduce_final(int count, const double *partial, double *out, cudaStream_t st, LaunchCounter &lc);
// One energy-trace entry of IBR_color: *dst = lambda (float)sums[0] + alpha (float)sums[1] (+ beta (float)sums[3]
// when grad), evaluated in float as the reference's host sums it (coco_vtv_sr_primal_energy_unstructured).
void launch_trace_energy(const double *sums, float lambda, float alpha, float beta, bool grad, double *dst,
                         cudaStream_t st, LaunchCounter &lc);
void launch_premultiply_dpart(int V, int n, const float *dpart3, int ch, float *dp, cudaStream_t st, LaunchCounter &lc);
void launch_copy_tau(int V, int n, const float *tau_in, int ch, float *tau, cudaStream_t st, LaunchCounter &lc);

// ---- push-pull (kernels_pushpull.cu)
// Pyramid buffers: img levels (3 channels each) and visibility levels, level s of size (W>>s) x (H>>s).
struct PushPull {
    float *img[11];
    uint8_t *vis[11];
    float *tmp;      // W x (H/2) x 3 scratch for the separable reduce/expand
    float *orig;     // 3 x N copy of the input (faithful "filled - U")
};
void launch_push_pull(int W, int H, bool faithful, const uint8_t *vis, float *U, PushPull &pp, cudaStream_t st,
                      LaunchCounter &lc);

// ---- IBR_gradient: hole filling and CG (kernels_cg.cu)
void launch_hole_fill_iter(int W, int H, const int *holes, int nholes, const float *Uin, float *Uout,
                           double *partial, cudaStream_t st, LaunchCounter &lc);
int hole_fill_partials(int nholes);
void launch_hole_list(int W, int H, const uint8_t *vis, int *holes, int *count, cudaStream_t st, LaunchCounter &lc);
void launch_cg_init(int W, int H, const float *U, const float *gx, const float *gy, float *r, float *d, bool faithful,
                    double *partial, cudaStream_t st, LaunchCounter &lc);
void launch_cg_apply(int W, int H, const float *d, float lambda, float *q, double *partial, cudaStream_t st,
                     LaunchCounter &lc);
void launch_cg_update(int W, int H, const float alpha[3], const float *d, const float *q, float *U, float *r,
                      double *partial, cudaStream_t st, LaunchCounter &lc);
void launch_cg_dir(int W, int H, const float beta[3], const float *r, float *d, cudaStream_t st, LaunchCounter &lc);
void launch_reduce_segments(int count, int nseg, const double *partial, double *out, cudaStream_t st, LaunchCounter &lc);
int cg_partials(int W, int H);

// Persistent (cooperative) solvers. The grid barrier's counter and error flag are zeroed before each launch;
// a barrier wait that exceeds its spin limit sets *err = 1 and the kernel returns.
struct GridBarrier {
    unsigned int *count;
    int *err;
};
int persistent_partials();  // upper bound of blocks (partials per slot)

// ---------------------------------------------------------------- corrected IBR_color (kernels_tv.cu)
constexpr int kTvInnerIterations = 200;  // FGP iterations per FISTA step (the oracle's kTvInner)
// Metric D = max(alpha sigma^2 sum_i A_i^T w_i, 1), the prox parameter lam = lambda / D and the dual step
// 1 / (8 max(lam_x, lam_{x+1}, lam_{x+W})) per target pixel.
void launch_tv_metric(const Geometry &G, const Buckets &B, const float *tau, const float *wgt, float as2, float lambda,
                      float *D, float *lam, float *linv, cudaStream_t st, LaunchCounter &lc);
// grad f = as2 sum_i A_i^T res_i (3 planes) from the splat-set residuals of launch_residual.
void launch_tv_gradf(const Geometry &G, const Buckets &B, const float *tau, const float *res, float as2, float *gf,
                     cudaStream_t st, LaunchCounter &lc);
// FP64 block partials of J_g(u), sum <grad u, p> and the box term of the certificate (c = gf - lambda div p; p FP64),
// three arrays of tv_gap_partials(W, H) entries each.
int tv_gap_partials(int W, int H);
void launch_tv_gap(int W, int H, const float *u, const float *gf, const double *P, const float *g, float lambda,
                   double *partial, cudaStream_t st, LaunchCounter &lc);
// Scalars of a corrected IBR_color solve whose loop runs on the device (a conditional graph): FISTA's t, the
// previous and current energy, the certified gap, steps taken, the stop and arithmetic flags, the non-finite flag,
// the energy trace's next slot, and the momentum weight theta of the next step.
struct TvLoopState {
    double t, E_prev, E, gap;
    int k, done, extended, err, trace_pos, pad;
    float theta;
};
// F = y - grad f(y) / D, y = u + theta (u - u_prev), grad f(y) = (1 + theta) gf - theta gf_prev (3 planes); theta
// from loop->theta when loop is given.
void launch_tv_fstep(int W, int H, const float *u, const float *up, const float *gf, const float *gfp, const float *D,
                     float theta, float *F, cudaStream_t st, LaunchCounter &lc, const TvLoopState *loop = nullptr);
// One thread: the energy and certified gap from the sums (slots 1, 4, 5, 6), the stop test (k >= niter or gap <=
// tol), and when going on the restart / momentum update, the switch to double-float below kTvExtendedBelow, and
// k + 1; sets h_loop to "go on" and h_extended to the arithmetic of the next step.
void launch_tv_decide(const double *sums, double dt_alpha, double lambda, double tol, int niter, TvLoopState *loop,
                      double *trace, int trace_cap, cudaGraphConditionalHandle h_loop,
                      cudaGraphConditionalHandle h_extended, cudaStream_t st, LaunchCounter &lc);
// out = clamp(in, 0, 1) over n floats.
void launch_tv_clamp(size_t n, const float *in, float *out, cudaStream_t st, LaunchCounter &lc);
// niter FGP iterations on the dual of the weighted ROF problem (one cooperative launch): P0 holds the starting
// dual (6 FP64 planes: x parts of the 3 channels, then the y parts) and receives the final one; P1, Q0, Q1 are
// scratch (6 FP64 planes each); U receives clamp(F + lam div p, 0, 1). extended: the dual's arithmetic in
// double-float (about 44 bits; else FP32), with the same FP64 storage.
// variant: the instantiation (iterations per super-step, block size) the autotuner picked; all give the same
// iterates (tv_fgp_variant_count per arithmetic; out of range: the default).
cudaError_t launch_tv_fgp(int W, int H, int niter, const float *F, const float *lam, const float *linv, const float *g,
                          double *P0, double *P1, double *Q0, double *Q1, float *U, GridBarrier gb, cudaStream_t st,
                          LaunchCounter &lc, bool extended, int variant = -1);
int tv_fgp_variant_count(bool extended);
int tv_fgp_default_variant(bool extended);
// The gap above which the FGP runs in FP32 (its certificate floor is near 4e-4): double-float takes over below it.
constexpr double kTvExtendedBelow = 2e-3;

// One target of a batched CG launch (k_cg_batch): its image, buffers and the contiguous range of blocks that
// work on it. state: [0..2] delta, [3] E, [4] gap, [5] iterations (written by the problem's first block).
struct CgProblem {
    int W, H, tiles_x, ntiles;
    int b0, nb;
    int max_iter;
    double gap_tol;
    const float *gx, *gy;
    float *U, *r, *dA, *dB;
    double *state;
    const float *U0;  // anchor when U holds a seed (nullptr: U is the anchor)
    double *trace;    // energy after each iteration (nullptr: none), at most trace_cap entries
    int trace_cap;
};
// Blocks of a batched launch: as many as can be resident with k_cg_batch's shape.
int cg_batch_resident_blocks();
cudaError_t launch_cg_batch(const CgProblem *d_probs, const int *d_block_prob, int nprob, int blocks, double *partA,
                            double *partB, int *done, GridBarrier gb, cudaStream_t st, LaunchCounter &lc);

// Persistent ROF instantiations (iterations per super-step x block size), chosen per image size by the host's
// autotuner; v indexes them.
int rof_variant_count();
int rof_default_variant();
int rof_persistent_steps(int niter, int v);
cudaError_t launch_rof_persistent(int W, int H, int niter, float tau, float sigma, float lam, float *U0, float *P0,
                                  float *U1, float *P1, const float *F, const float *g, GridBarrier gb, int v,
                                  cudaStream_t st, LaunchCounter &lc);
// poisson_jacobi (sources/gradientIBR.cu:923-1013): `iters` Jacobi sweeps on U (3 planes) in one cooperative launch;
// U1 (3 planes), z (3 planes) and den (1 plane) are scratch.
cudaError_t launch_poisson_jacobi(int W, int H, int iters, const float *gx, const float *gy, const float *mask,
                                  float *U, float *U1, float *z, float *den, GridBarrier gb, cudaStream_t st,
                                  LaunchCounter &lc);
cudaError_t launch_cg_persistent(int W, int H, const float *gx, const float *gy, float *U, float *r, float *dA,
                                 float *dB, double *partA, double *partB, GridBarrier gb, int max_iter, double gap_tol,
                                 double *state, cudaStream_t st, LaunchCounter &lc, const float *U0 = nullptr,
                                 double *trace = nullptr, int trace_cap = 0);
cudaError_t launch_hole_fill_persistent(int W, int H, const int *holes, const int *count, float *A, float *B,
                                        double *part, GridBarrier gb, int max_iter, double *state, cudaStream_t st,
                                        LaunchCounter &lc);
void launch_cg_energy(int W, int H, const float *U, const float *U0, const float *gx, const float *gy, double *partial,
                      cudaStream_t st, LaunchCounter &lc);

// ------------------------------------------------------------------ learned warm start (tcgen05 convolutions)
// Implicit-GEMM convolution: rows are the batch x Ho x Wo pixels of the output (forward) or of the forward input
// (dgrad); the gathered tensor src is NHWC BF16 with C channels over batch x Hs x Ws; B is the BF16 weight matrix
// [N][ldw] (K contiguous, zero padded to ldw, a multiple of 64). Epilogue: + bias, + add, ReLU, zero where
// mask <= 0; outputs [rows][N] in FP32 and/or BF16.
struct ConvGemm {
    const void *src;
    int C, Hs, Ws;
    int batch, Ho, Wo;
    int ks, stride, dgrad;
    int K;
    const void *wt;
    int ldw, N;
    const float *bias;
    int relu;
    const void *add, *mask;
    float *outf;
    void *outb;
    // nearest-upsampling fusion (1 x 1 decoder layers): with upskip set, each output pixel's value v is written as
    // relu(v + upskip) to its 2 x 2 block of outb at (2 Ho) x (2 Wo), upskip being a BF16 tensor of that size
    const void *upskip;
};
// Weight gradient of a convolution with input x (Cin channels, Hx x Wx) and output gradient dy (Cout stored
// channels, Ho x Wo): rows (tap, ci) of dW^T padded to Mpad, the pixels split into chunks (a multiple of 64),
// FP32 partial[split][Mpad][Cout].
struct WgradGemm {
    const void *x;
    int Cin, Hx, Wx;
    const void *dy;
    int Cout, Ho, Wo;
    int batch, ks, stride;
    int Kf, Mpad, chunk;
    float *partial;
};
cudaError_t launch_conv_tc(const ConvGemm &g, int *err, cudaStream_t st, LaunchCounter &lc);
// Kernel choice of launch_conv_tc: 0 TMA / resident tile / gather as they apply, 1 without the TMA kernel, 2 the
// gather kernel only (process-wide).
void set_conv_kernel_pref(int pref);
cudaError_t launch_wgrad_tc(const WgradGemm &g, int splits, int Cout_real, float *grad, int *err, cudaStream_t st,
                            LaunchCounter &lc);
cudaError_t launch_bias_grad(int P, int C, int Creal, const void *dy, float *partial, int blocks, float *out,
                             cudaStream_t st, LaunchCounter &lc);
cudaError_t launch_upsample_add_relu(int batch, int Hl, int Wl, int C, const void *t, const void *skip, void *s,
                                     cudaStream_t st, LaunchCounter &lc);
cudaError_t launch_down_sum(int batch, int Hl, int Wl, int C, const void *ds, void *dt, cudaStream_t st,
                            LaunchCounter &lc);
cudaError_t launch_output_head(int batch, int HW, int Cy, const float *y, const float *u0, const float *target,
                               float *pred, void *dy, double *loss_partial, int blocks, cudaStream_t st,
                               LaunchCounter &lc);
cudaError_t launch_adam(size_t n, float *w, const float *grad, float *m, float *v, float lr_t, float b1, float b2,
                        float eps_t, cudaStream_t st, LaunchCounter &lc);
cudaError_t launch_pack_weights(int Cout, int Cst, int Cin, int taps, int Kpad, int Kdpad, const float *w, void *Wb,
                                void *Wt, cudaStream_t st, LaunchCounter &lc);

}  // namespace lfrv
