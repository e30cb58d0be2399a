/* lfrv.h -- C ABI of the GB300 light-field remote-vision solver library (liblfrv.so).
 *
 * The reference (Nighteye/light-field-remote-vision) has no plugin or FFI layer: its hot path is
 * reached through the config-driven C++ entry points
 *     void sr_synthesize_view( Config_data*, int frame )      sources/super-resolution.h:12
 *     void IBR_gradient( Config_data* )                       sources/gradientIBR.h:7
 * and the cocolib-style stage functions coco_vtv_sr_*_unstructured( coco_vtv_data* )
 * (sources/optimization.cuh:111-175), which allocate and free all device memory themselves, run on
 * the default stream and assert() on any error (cocolib/cocolib/cuda/cuda_helper.h:38-44).
 *
 * This header replaces that boundary with plain C:
 *   - every entry point returns an int status: LFRV_OK (0) or a negative LFRV_E_* code;
 *     lfrv_last_error() returns a message for the calling thread's last failure;
 *   - images are planar float32, channel-major (C x H x W), row-major, top-left origin;
 *     per-view stacks are V x C x h x w in the order of the reference's import loops
 *     (s = s_min..s_max skipping s_rmv, sources/import.cpp:144-160);
 *   - host entry points take caller-owned host buffers and copy them in/out; *_dev entry points take
 *     caller-owned device pointers and a cudaStream_t (passed as void*), and never synchronise the
 *     device beyond that stream;
 *   - a context (lfrv_ctx) owns the device workspace of one solve; contexts are independent, so
 *     distinct threads may drive distinct contexts concurrently.
 */
#ifndef LFRV_H
#define LFRV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define LFRV_OK              0
#define LFRV_E_ARG          -1   /* bad argument (null pointer, size mismatch, unsupported option) */
#define LFRV_E_CUDA         -2   /* a CUDA runtime call or kernel launch failed */
#define LFRV_E_NOMEM        -3   /* device or host allocation failed */
#define LFRV_E_IO           -4   /* file could not be opened, read or written */
#define LFRV_E_FORMAT       -5   /* malformed file (PFM header, config syntax) */
#define LFRV_E_NONFINITE    -6   /* non-finite value in an input or in the solver state */
#define LFRV_E_TIMEOUT      -7   /* a bounded device-side wait gave up */
#define LFRV_E_NODEVICE     -8   /* no CUDA device, or the library was built without a usable kernel image */

const char *lfrv_last_error(void);
const char *lfrv_version(void);

/* ---------------------------------------------------------------- configuration
 * Mirrors the keys of Config_data (sources/config.h:11-122, parsed in sources/config.cpp:67-129) that
 * the IBR_color / IBR_gradient path reads, with the reference's defaults (sources/config.cpp:11-64).
 * sigma_sensor holds the value AFTER the reference's division by 255 (sources/config.cpp:119).
 */
typedef struct lfrv_config {
    int   w, h;              /* input (low-res) view size                       ("width", "height") */
    int   dsf;               /* super-resolution factor; target is (dsf*w) x (dsf*h)        ("dsf") */
    int   nviews;            /* number of input views (all views but s_rmv)                         */
    int   nchannels;         /* must be 3 (sources/config.cpp:116)                                  */
    float sigma_sensor;      /* sensor noise sigma, already divided by 255                          */
    float ugrad_threshold;   /* clamp of the warped target gradient in the angular weights         */
    float lambda;            /* TV smoothness                                                       */
    float lambda_max_factor; /* lambda_max = lambda_max_factor * lambda in the regulariser weight   */
    int   dw_type;           /* deformation weights: only 0 (Wanner) is implemented upstream        */
    int   gw_type;           /* gradient-term weights (energy of the gradient data term)            */
    float dt_alpha;          /* intensity data term weight                                          */
    float dt_beta;           /* gradient data term weight                                           */
    float gradient_step;     /* step of the gradient data term                                      */
    int   niter;             /* outer FISTA iterations AND inner ROF iterations (reference reuses it); in
                                corrected IBR_color (faithful = 0) the cap on outer FISTA steps */
    int   nmeta_iter;        /* re-weighting meta iterations                                         */
    /* --- options with no Config_data counterpart --- */
    int   faithful;          /* 1: reproduce the reference's control flow including its defects      */
    int   early_exit;        /* 1: the reference's convergence tests (energy / moving pixels) apply  */
    int   cg_max_iter;       /* IBR_gradient, corrected CG: iteration cap                             */
    double cg_gap_tol;       /* corrected mode (faithful = 0): stop when the certified relative energy gap falls
                                to this value (0: run the cap). IBR_gradient: ||r||^2 / (2 lambda_cg) / |E(u)| of
                                the CG. IBR_color: the primal-dual gap of the weighted TV_F objective over E(u)
                                (kernels_tv.cu's certificate) */
    int   hole_fill_iter;    /* IBR_gradient hole filling: Jacobi iteration cap (reference: 500)     */
    int   bf16_storage;      /* IBR_gradient, device entry points: 1 = d_views holds BF16 values (V x 3 x h x w
                                bfloat16), and the view gradients and weights are stored in BF16 too; every
                                accumulation stays FP32 and the CG's dot products and energy FP64 (default 0) */
} lfrv_config;

/* Fills *cfg with Config_data's defaults (sources/config.cpp:11-64) and this library's option defaults
 * (faithful=1, early_exit=1, cg_max_iter=500, cg_gap_tol=1e-4, hole_fill_iter=500). */
int lfrv_config_default(lfrv_config *cfg);

/* Parses a reference config file (coco::config syntax: "key value" lines, '#' comments,
 * "config <file>" includes processed in order, later keys override; cocolib/cocolib/common/
 * parse_config.cpp:44-200) into *cfg, applying sigma_sensor /= 255 as Config_data::parse_config does.
 * String-valued keys the solver needs (lf_name, tau_name, dpart_name, init_name, outdir, outfile,
 * algorithm) are returned through lfrv_config_get_string after the call. s_min/s_max/s_rmv set nviews. */
int lfrv_config_parse_file(const char *path, lfrv_config *cfg);
int lfrv_config_set(lfrv_config *cfg, const char *key, const char *value);
int lfrv_config_get_string(const char *key, char *buf, size_t buflen);
int lfrv_config_get_int(const char *key, int *value);

/* ---------------------------------------------------------------- cameras
 * Pinhole P = K [R | t], t = -R C (sources/pinholeCamera.h:14-57). Row-major 3x3 K and R. */
typedef struct lfrv_camera {
    float K[9];
    float R[9];
    float t[3];
    int   width, height;
} lfrv_camera;

/* ---------------------------------------------------------------- solve statistics */
typedef struct lfrv_stats {
    int    outer_iterations;     /* FISTA iterations run (IBR_color) or CG iterations (IBR_gradient) */
    int    meta_iterations;
    int    hole_fill_iterations;
    int    stop_reason;          /* 0 cap reached, 1 tiny energy, 2 relative energy change, 3 < 1% pixels moving,
                                    4 certified gap reached */
    double energy;               /* last energy evaluated: the reference formula for IBR_color (faithful), the TV_F
                                    objective (corrected IBR_color), the quadratic energy for CG */
    double gap;                  /* last certified relative gap (corrected modes), else 0 */
    double seconds;              /* device time of the solve (CUDA events) */
    int    kernel_launches;      /* kernels this library launched for the call */
    /* Optional energy trace (the reference prints the energy of every FISTA iteration,
     * sources/super-resolution.cpp:221-260). The caller sets energy_trace to a host buffer of trace_capacity
     * doubles (or NULL / 0 for none) before the call; the solver writes one entry per outer iteration, in order:
     * IBR_color (faithful): the energy of coco_vtv_sr_primal_energy_unstructured (sources/optimization.cu:1477-1717)
     * after each FISTA iteration, across meta iterations; corrected IBR_color: the TV_F objective of the starting
     * point and of every FISTA iterate; IBR_gradient: the quadratic energy
     * 1/2 ||u - u0||^2 + 1/2 ||grad u - g||^2 after each CG iteration (FP64). trace_length receives the number of
     * entries written (at most trace_capacity). Zero-initialise the struct: the library reads these two fields. */
    double *energy_trace;
    int    trace_capacity;
    int    trace_length;
} lfrv_stats;

/* ---------------------------------------------------------------- contexts */
typedef struct lfrv_ctx lfrv_ctx;

int lfrv_ctx_create(lfrv_ctx **out, int device);
int lfrv_ctx_destroy(lfrv_ctx *ctx);
/* All device work of the context is issued on this stream (a cudaStream_t; NULL = legacy default). */
int lfrv_ctx_set_stream(lfrv_ctx *ctx, void *cuda_stream);
/* Counts kernels launched by the context since creation (or the last reset). */
int lfrv_ctx_launch_count(lfrv_ctx *ctx, long long *count, int reset);
/* Per-kernel device timing (no counterpart upstream; the reference prints iter/s from clock(),
 * sources/super-resolution.cpp:266-270). enable=1 clears the records and records a CUDA event pair on the
 * context stream around every kernel launch (when its pool of 16384 pairs fills, the stream is synchronised
 * and the pairs are folded into per-kernel totals, so profiling mode adds host waits between launches);
 * lfrv_ctx_profile_read synchronises the stream and returns, for the index-th kernel name seen, its summed
 * device time and launch count (LFRV_E_ARG past the end). */
int lfrv_ctx_profile(lfrv_ctx *ctx, int enable);
int lfrv_ctx_profile_read(lfrv_ctx *ctx, int index, char *name, size_t name_len, double *total_ms,
                          long long *launches);

/* ---------------------------------------------------------------- depth maps
 * Radial to orthographic depth, in place (fromRadial2Ortho.frag:10-23, applied by InputView::filterDepthmap,
 * sources/openGL/view.cpp:723-733, to MVE depth maps): depth is nviews x 3 x h x w (z, dz/dx, dz/dy); with
 * X = K^-1 (x + 1/2, y + 1/2, 1) and d = |X| the result is z / d and its derivatives
 * dz/dx / d - z (X . K^-1 column 0) / d^3 (column 1 for y). Only K of each camera is used. */
int lfrv_depth_radial_to_ortho(lfrv_ctx *ctx, int nviews, int w, int h, const lfrv_camera *cams, float *depth);
int lfrv_depth_radial_to_ortho_dev(lfrv_ctx *ctx, int nviews, int w, int h, const lfrv_camera *cams,
                                   float *d_depth);

/* Warps from orthographic depth maps and cameras without the GL pipeline: import_warps_from_depth
 * (sources/import.cpp:243-450), the path sr_synthesize_view and IBR_gradient take when a config names depth
 * maps and cameras (sources/super-resolution.cpp:121-127, sources/gradientIBR.cpp:62-68).
 * - depth is nviews x depth_channels x h x w; plane 0 holds z.
 * - tau (nviews x 3 x h x w) receives tau_x, tau_y, tau_y, as the reference writes it.
 * - Pixels whose depth is outside [1/1000, 1000], or that have no target coverage, get (-w, -h).
 * - Pixels whose back-projection lands more than 10 pixels from the source pixel get (-2w, -2h).
 * - faithful = 1 back-projects with the source view's R and C as the reference does (import.cpp:412-415).
 *   faithful = 0 uses the target's. */
int lfrv_warp_from_depth(lfrv_ctx *ctx, int nviews, int w, int h, int dsf, const float *depth, int depth_channels,
                         const lfrv_camera *cams, const lfrv_camera *target, int faithful, float *tau);
int lfrv_warp_from_depth_dev(lfrv_ctx *ctx, int nviews, int w, int h, int dsf, const float *d_depth,
                             int depth_channels, const lfrv_camera *cams, const lfrv_camera *target, int faithful,
                             float *d_tau);

/* ---------------------------------------------------------------- warp stage
 * Replaces the GL warp exporter (fromMVE2coco: Scene::computeTargetDepthMap sources/openGL/scene.cpp:1506,
 * Scene::exportWarps :1546, shaders tauWarp.frag:25-74, tauPartial.frag:23-48,
 * depthSplatting.{vert,geom,frag}) with CUDA kernels writing headless device buffers.
 *   depth   : V x 3 x h x w   (z, dz/dx, dz/dy) per input view, orthographic depth along the optical axis
 *   cams    : V input cameras; target: the target camera (target->width x target->height = W x H)
 *   tau     : V x 3 x h x w   (tau_x, tau_y, deformation weight), codes -2 / -1 as tauWarp.frag writes
 *   dpart   : V x 3 x h x w   (sigma_z = 10, dtau_x/dz, dtau_y/dz) as tauPartial.frag writes
 *   zbuf    : H x W            target depth map (0 where no quad covers a pixel centre), may be NULL
 */
int lfrv_warp(lfrv_ctx *ctx, int nviews, int w, int h,
              const float *depth, const lfrv_camera *cams, const lfrv_camera *target,
              float *tau, float *dpart, float *zbuf);
int lfrv_warp_dev(lfrv_ctx *ctx, int nviews, int w, int h,
                  const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target,
                  float *d_tau, float *d_dpart, float *d_zbuf);

/* ---------------------------------------------------------------- solvers
 * lfrv_ibr_color replaces sr_synthesize_view (sources/super-resolution.cpp:54-338);
 * lfrv_ibr_gradient replaces IBR_gradient (sources/gradientIBR.cpp:12-150).
 *   views : V x 3 x h x w input views (the reference's view_data::_image_f)
 *   tau   : V x 2 x h x w or V x 3 x h x w warps; only channels 0,1 are read (coco_vtv_sr_read_tau,
 *           sources/optimization.cu:1170-1205, ignores the deformation channel)
 *   dpart : V x 3 x h x w (sigma_z, dtau_x/dz, dtau_y/dz); the solver uses sigma_z*dtau/dz
 *           (coco_vtv_sr_read_partial_tau, sources/optimization.cu:1208-1256)
 *   init  : optional 3 x H x W starting image (the reference's init_name PFM), NULL = computed
 *   out   : 3 x H x W result
 * tau_stride_ch selects the channel count of the tau stack (2 or 3).
 */
int lfrv_ibr_color(lfrv_ctx *ctx, const lfrv_config *cfg,
                   const float *views, const float *tau, int tau_channels, const float *dpart,
                   const float *init, float *out, lfrv_stats *stats);
int lfrv_ibr_color_dev(lfrv_ctx *ctx, const lfrv_config *cfg,
                       const float *d_views, const float *d_tau, int tau_channels, const float *d_dpart,
                       const float *d_init, float *d_out, lfrv_stats *stats);
int lfrv_ibr_gradient(lfrv_ctx *ctx, const lfrv_config *cfg,
                      const float *views, const float *tau, int tau_channels, const float *dpart,
                      const float *init, float *out, lfrv_stats *stats);
int lfrv_ibr_gradient_dev(lfrv_ctx *ctx, const lfrv_config *cfg,
                          const float *d_views, const float *d_tau, int tau_channels, const float *d_dpart,
                          const float *d_init, float *d_out, lfrv_stats *stats);

/* Full depth-to-image pipeline on one target: the warp stage (fromMVE2coco's GL export,
 * sources/openGL/scene.cpp:1506-1586) followed by the solver (algorithm 0 = IBR_color as
 * sr_synthesize_view, 1 = IBR_gradient as IBR_gradient), as the reference's IBR_video loop chains them
 * per frame (sources/main.cpp:359-403). views and depth are V x 3 x h x w; out is 3 x H x W.
 * lfrv_render_view takes host buffers (copied in and out inside the call); _dev takes device pointers. */
int lfrv_render_view(lfrv_ctx *ctx, const lfrv_config *cfg, int algorithm,
                     const float *views, const float *depth,
                     const lfrv_camera *cams, const lfrv_camera *target,
                     float *out, lfrv_stats *stats);
int lfrv_render_view_dev(lfrv_ctx *ctx, const lfrv_config *cfg, int algorithm,
                         const float *d_views, const float *d_depth,
                         const lfrv_camera *cams, const lfrv_camera *target,
                         float *d_out, lfrv_stats *stats);

/* ---------------------------------------------------------------- batched targets
 * No single reference counterpart: the reference renders one target per process run (main, sources/main.cpp:
 * 349-357). A batch renders many target views, each with its own light field, sizes and options, on device
 * buffers and the context's stream. IBR_gradient jobs with faithful = 0 run warp, set-up and hole filling one
 * after another, then share one persistent CG launch (k_cg_batch) in which every job keeps its own tiles,
 * dot products, stop rule and statistics; other jobs run as lfrv_render_view_dev would. The call returns when
 * every output is written. */
typedef struct lfrv_view_job {
    const lfrv_config *cfg;    /* sizes (w, h, dsf, nviews) and solver options of this target */
    int algorithm;             /* 0 IBR_color, 1 IBR_gradient */
    const float *d_views;      /* nviews x 3 x h x w, device */
    const float *d_depth;      /* nviews x 3 x h x w (z, dz/dx, dz/dy), device */
    const lfrv_camera *cams;   /* nviews input cameras, host */
    const lfrv_camera *target; /* host */
    float *d_out;              /* 3 x H x W, device */
    lfrv_stats *stats;         /* optional */
} lfrv_view_job;
int lfrv_render_views_dev(lfrv_ctx *ctx, const lfrv_view_job *jobs, int count);
/* The same batch from HOST buffers: each job's d_views, d_depth and d_out are host pointers (views BF16 when the
 * job's cfg->bf16_storage is 1). Input buffers shared by several jobs (same pointer and size, e.g. one light field
 * seen from many targets) are uploaded once, the colour views while the warp stage runs. An IBR_gradient job's
 * output in pinned (page-locked) host memory is copied back as soon as its CG ends, while later jobs run; every
 * output is in host memory when the call returns. */
int lfrv_render_views(lfrv_ctx *ctx, const lfrv_view_job *jobs, int count);

/* ---------------------------------------------------------------- IBR_video
 * The reference's IBR_video loop (sources/main.cpp:359-403) renders frame after frame of one light field from a
 * moving target camera (TargetView::move, sources/openGL/view.cpp:1744-1759): the centre goes from input view a's
 * towards view b's by frame / 1000 of the way and the rotation is view a's turned about the y axis by frame * 0.0003
 * rad (the reference takes views 5 and 3); K and the size stay the target's.
 * lfrv_video_camera: that camera for one frame. lfrv_render_video_dev: frames first_frame .. first_frame + nframes - 1
 * rendered as one batch (as lfrv_render_views_dev); d_out holds nframes x 3 x H x W, stats (optional) nframes entries. */
int lfrv_video_camera(const lfrv_camera *a, const lfrv_camera *b, const lfrv_camera *target, int frame,
                      lfrv_camera *out);
int lfrv_render_video_dev(lfrv_ctx *ctx, const lfrv_config *cfg, int algorithm, const float *d_views,
                          const float *d_depth, const lfrv_camera *cams, int cam_a, int cam_b,
                          const lfrv_camera *target, int first_frame, int nframes, float *d_out, lfrv_stats *stats);

/* ---------------------------------------------------------------- learned warm start
 * No reference counterpart: an addition beside the plain method, which stays unchanged. A 4-scale
 * encoder-decoder convolutional network (~1.23 M parameters, BF16 weights and activations, FP32 accumulation
 * on the tensor cores, FP32 master weights and Adam state) predicts the converged IBR_gradient solution from
 * LFRV_WARMSTART_CHANNELS per-pixel inputs; the prediction only seeds the CG iterate of the corrected solver
 * (faithful = 0). The anchor u0 of the normal equations (lambda I - Delta) u = lambda u0 + grad^T g
 * (sources/solver.cu:526-699) stays the hole-filled weighted average, so the solution, the energy and the
 * certified-gap stop are those of the plain solver: a poor prediction costs iterations, never accuracy.
 * Targets (H, W) must be multiples of 8.
 *
 * Input channels (NHWC BF16, per target pixel): [0..2] u0, [3] gx, [4] gy (the luminance gradient constraint,
 * zero in the last column / row, clamped to [-1, 1]), [5] visibility, [6 + 3v .. 8 + 3v] view v splatted alone,
 * [30 + v] view v's share of the splat weight (views v < 8), [38..40] the CG's initial residual at u0
 * (grad^T g + Delta u0 per channel, clamped to [-4, 4]), [41..47] zero. Parameters (lfrv_warmstart_get_params):
 * flat FP32, per layer W[cout][ky][kx][cin] then
 * bias[cout], layers in the order of the network description in learn.cpp. */
#define LFRV_WARMSTART_CHANNELS 48
typedef struct lfrv_warmstart lfrv_warmstart;
long long lfrv_warmstart_param_count(void);
int lfrv_warmstart_create(lfrv_ctx *ctx, unsigned long long seed, lfrv_warmstart **net);
void lfrv_warmstart_destroy(lfrv_warmstart *net);
int lfrv_warmstart_get_params(lfrv_warmstart *net, float *params);
int lfrv_warmstart_set_params(lfrv_warmstart *net, const float *params);  /* also resets the Adam state */
/* Training data of one target: the network input (H x W x 48 BF16), the anchor u0 (3 x H x W) and, when
 * d_solution is not NULL, the plain solver's solution from u0 to cfg->cg_gap_tol (3 x H x W). */
int lfrv_warmstart_features_dev(lfrv_ctx *ctx, const lfrv_config *cfg, const float *d_views,
                                const float *d_depth, const lfrv_camera *cams, const lfrv_camera *target,
                                void *d_input, float *d_u0, float *d_solution, lfrv_stats *stats);
/* Batched tensors: input batch x H x W x 48 (BF16), u0 / target / prediction batch x 3 x H x W (FP32). */
int lfrv_warmstart_forward_dev(lfrv_warmstart *net, int batch, int H, int W, const void *d_input,
                               const float *d_u0, float *d_pred);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on the mean squared error of u0 + net(input) against target;
 * *loss = the loss before the step. */
int lfrv_warmstart_train_step_dev(lfrv_warmstart *net, int batch, int H, int W, const void *d_input,
                                  const float *d_u0, const float *d_target, float lr, double *loss);
/* Loss and its gradient with respect to every parameter (host, lfrv_warmstart_param_count floats), no update. */
int lfrv_warmstart_gradients_dev(lfrv_warmstart *net, int batch, int H, int W, const void *d_input,
                                 const float *d_u0, const float *d_target, double *loss, float *grads);
/* IBR_gradient of one target (as lfrv_render_view_dev with algorithm 1) with the CG seeded by the network. */
int lfrv_render_view_warm_dev(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_config *cfg,
                              const float *d_views, const float *d_depth, const lfrv_camera *cams,
                              const lfrv_camera *target, float *d_out, lfrv_stats *stats);
/* Batched targets (as lfrv_render_views_dev) with every IBR_gradient job of faithful = 0 and a target of
 * multiples of 8 pixels seeded by the network, which must belong to ctx: the jobs' inputs are built on the helper
 * lanes with their set-up, the network predicts each seed on the context stream, and the shared CG launch starts
 * every seeded job from its prediction with its own anchor. */
int lfrv_render_views_warm_dev(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_view_job *jobs, int count);
/* lfrv_render_views_warm_dev from host buffers, as lfrv_render_views. */
int lfrv_render_views_warm(lfrv_ctx *ctx, lfrv_warmstart *net, const lfrv_view_job *jobs, int count);
/* One convolution through the tensor-core kernels: x NHWC BF16 (batch x H x W x Cin), dy NHWC BF16
 * (batch x H/stride x W/stride x Cout), w FP32 Cout x ks x ks x Cin (rounded to BF16 inside), out FP32.
 * mode 0: out = conv(x) (batch x H/s x W/s x Cout); 1: out = the data gradient (batch x H x W x Cin);
 * 2: out = the weight gradient (Cout x ks x ks x Cin). ks 1 or 3 (padding 1), stride 1 or 2, Cin a multiple of
 * 8, Cout (and Cin for mode 1) one of 16, 32, 64, 128, 256. */
int lfrv_conv_bf16_dev(lfrv_ctx *ctx, int mode, int batch, int H, int W, int Cin, int Cout, int ks, int stride,
                       const void *d_x, const void *d_dy, const float *d_w, float *d_out);
/* Which tensor-core convolution kernels the network's layers may use (process-wide; all give the same results to
 * within FP32 summation order): 0 (default) the TMA-fed kernel where its 128-pixel patch tiling applies, else
 * the resident-tile kernel (stride-1 3 x 3 on rows of a multiple of 128), else the cp.async gather; 1 the last
 * two; 2 the gather only. */
int lfrv_set_conv_kernel(int which);

/* ---------------------------------------------------------------- stage calls
 * Fine-grained entry points mirroring the cocolib stage functions, used by the parity tests.
 * All take host buffers. "views/tau/dpart" as above; U, G etc. are 3 x H x W.
 */
/* coco_vtv_sr_compute_weights_unstructured (sources/optimization.cu:1066-1167) with the reference's
 * buffer semantics: gx/gy (H x W) are the gradient buffers the Sobel kernel writes (X1[0], X2[0]) and
 * keep their old value where the kernel does not write; vis (H x W bytes) the visibility mask.
 * Writes weights (V x h x w). */
int lfrv_stage_weights(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                       int tau_channels, const float *dpart, const float *U, const uint8_t *vis,
                       float *gx, float *gy, float *weights);
/* coco_vtv_setup_visibility_mask (sources/optimization.cu:33-135): coverage (H x W) and vis (H x W). */
int lfrv_stage_visibility(lfrv_ctx *ctx, const lfrv_config *cfg, const float *tau, int tau_channels,
                          float *coverage, uint8_t *vis);
/* vtv_sr_dataterm_intensities + the F computation of vtv_sr_ista_step_unstructured
 * (sources/optimization.cu:1751-1812, 1835-1966): G (3 x H x W, before the [-1,1] clamp) and
 * F = clamp(U - clamp(G,-1,1)/(lambda L), 0, 1). */
int lfrv_stage_dataterm(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                        int tau_channels, const float *weights, const float *U, float *G, float *F);
/* niter inner ROF iterations (sources/optimization.cu:1815-1828; vtv_rof.cu:118-147, 280-320;
 * cuda_kernels.cu:504-532) in place on U (3 x H x W) and the duals P (6 x H x W: px0,py0,px1,py1,px2,py2)
 * for data F (3 x H x W) and regulariser weight g (H x W). */
int lfrv_stage_rof(lfrv_ctx *ctx, int W, int H, int niter, float tau, float sigma, float lambda,
                   const float *F, const float *g, float *U, float *P);
/* Reference energy (coco_vtv_sr_primal_energy_unstructured, sources/optimization.cu:1477-1717). */
int lfrv_stage_energy(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                      int tau_channels, const float *weights, const float *U, const uint8_t *vis,
                      double *energy, double *e_tv, double *e_data);
/* Regulariser weight g (H x W) (coco_vtv_sr_init_regularizer_weight_unstructured,
 * sources/optimization.cu:2251-2338). norm_in is the coverage accumulator's prior content
 * (the reference never clears it here); norm_out receives its final content. */
int lfrv_stage_regularizer(lfrv_ctx *ctx, const lfrv_config *cfg, const float *tau, int tau_channels,
                           const float *weights, const float *norm_in, float *norm_out, float *g);
/* Weighted-average initial image before hole filling (coco_vtv_sr_compute_initial_image,
 * sources/optimization.cu:1300-1350): U (3 x H x W) and the weight sum norm (H x W). */
int lfrv_stage_initial_image(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                             int tau_channels, const float *weights, float *U, float *norm);
/* Push-pull hole filling (coco_vtv_push_pull, sources/optimization.cu:544-651) in place on U
 * (3 x H x W) with visibility vis; faithful=1 reproduces the reference's final "U = filled - U". */
int lfrv_stage_push_pull(lfrv_ctx *ctx, int W, int H, int faithful, const uint8_t *vis, float *U);
/* IBR_gradient pieces: splat visibility (setup_target_visibility, sources/gradientIBR.cu:40-83),
 * Laplacian hole filling (hole_filling, :87-152), gradient splatting (init_u_gradient, :833-920)
 * and the Poisson CG (possion_conj_grad, sources/solver.cu:526-699). */
int lfrv_stage_gradient_visibility(lfrv_ctx *ctx, const lfrv_config *cfg, const float *tau,
                                   int tau_channels, uint8_t *vis);
int lfrv_stage_hole_fill(lfrv_ctx *ctx, int W, int H, int max_iter, const uint8_t *vis, float *U,
                         int *iterations);
int lfrv_stage_u_gradient(lfrv_ctx *ctx, const lfrv_config *cfg, const float *views, const float *tau,
                          int tau_channels, const float *weights, float *gx, float *gy, float *mask);
/* faithful=1: the reference's 5-iteration loop with its defects; faithful=0: conjugate gradient with
 * FP64 dot products until the certified gap reaches gap_tol or max_iter iterations. */
int lfrv_stage_cg(lfrv_ctx *ctx, int W, int H, int faithful, int max_iter, double gap_tol,
                  const float *gx, const float *gy, float *U, int *iterations, double *gap);

/* poisson_jacobi (sources/gradientIBR.cu:923-1013), the Jacobi alternative to the CG that IBR_gradient leaves
 * commented out (sources/gradientIBR.cpp:131): z = (m u0 - div g) / (4 + m) per channel with the central-difference
 * divergence of (gx, gy), then `iterations` sweeps (200 upstream) u <- (sum of the 4 neighbours, the border pixel
 * repeated) / (4 + m) + z. gx, gy, mask: H x W; U: 3 x H x W (in: u0, out: the result). All sweeps run in one
 * persistent launch. */
int lfrv_stage_poisson_jacobi(lfrv_ctx *ctx, int W, int H, int iterations, const float *gx, const float *gy,
                              const float *mask, float *U);

/* Allocation-free corrected CG. No reference counterpart.
 * The same solver as lfrv_stage_cg with faithful = 0, on caller-owned DEVICE buffers on `stream`
 * (a cudaStream_t of the current device, or NULL for the legacy default stream): gx, gy are H x W,
 * U is 3 x H x W (in: u0, out: the solution).
 * All of its scratch sits in one fixed device array built into the library. That array holds r and two
 * direction buffers, the FP64 block partials, the solver state and the grid-barrier words. It is about
 * 9.5 MB per device, for W * H <= LFRV_CG_STATIC_MAX_PIXELS. No call allocates or frees device memory,
 * and none creates a context or a stream: this is the entry point for callers that cannot allocate.
 * - Larger images are rejected with LFRV_E_ARG, before any device work.
 * - First call on a device (per driver context of that device): it looks up the array's address with the
 *   device current, and later calls reuse it. Under lazy module loading (CUDA's default since 12.2) that first
 *   lookup also loads the library's device code and so reserves the array's memory on the device: make one call
 *   (any valid size) during start-up, outside the section that must not allocate and before any stream capture
 *   that includes the call. Setting CUDA_MODULE_LOADING=EAGER loads it when the context is created instead.
 *   After cudaDeviceReset, or under another context of the same device, the address is looked up again.
 * - The barrier words are cleared on `stream` before each launch. Nothing else needs to start at zero.
 * - There is one array per device. Calls that overlap on the same device race on it, even from different
 *   streams or threads. Order such calls, for example on one stream.
 * - With iterations or gap non-NULL the call synchronises `stream` and reads the iteration count, the
 *   certified gap and the barrier status (LFRV_E_TIMEOUT). With both NULL it only enqueues work. */
#define LFRV_CG_STATIC_MAX_PIXELS (512 * 512)
int lfrv_cg_solve_static(void *stream, int W, int H, int max_iter, double gap_tol, const float *gx,
                         const float *gy, float *U, int *iterations, double *gap);

/* ---------------------------------------------------------------- files
 * PFM as the reference reads and writes it: gsl_image_load_pfm (cocolib/cocolib/common/gsl_image.cpp:
 * 416-500) flips rows on load; write_pfm_image_signed (cocolib/cocolib/cuda/cuda_helper.cu:340-375)
 * flips on write. Buffers here are top-left origin, planar. */
int lfrv_pfm_read(const char *path, int *w, int *h, int *channels, float *data, size_t capacity);
int lfrv_pfm_write(const char *path, int w, int h, int channels, const float *data);
/* MVE depth and normal maps (InputView::importMVEIFile, sources/openGL/view.cpp:279-325): a text header line, then
 * width, height, channels, type as four little-endian uint32, then interleaved float32 pixels, row 0 first; returned
 * planar (channels x h x w). A NULL data pointer returns only the sizes. */
int lfrv_mvei_read(const char *path, int *w, int *h, int *channels, float *data, size_t capacity);
/* InputView::setDepthAndNormals (sources/openGL/view.cpp:607-635) with Texture::loadFromData (sources/openGL/
 * texture.cpp:207-290): the depth plane (h0 x w0) and the first two normal planes (2 x h0 x w0) become the three
 * depth-map channels (out: 3 x h0*factor x w0*factor), upsampled by nearest neighbour; pixels whose three values are
 * all 0 become (invalid_depth, 0, 0) (the reference uses INVALID_DEPTH = 1000). Feed the result to
 * lfrv_depth_radial_to_ortho, as Scene::filterDepthMaps does. */
int lfrv_depth_from_mve(int w0, int h0, int factor, const float *depth, const float *normal, float invalid_depth,
                        float *out);
/* 8-bit PNG as gsl_image_load / gsl_image_save read and write it through Qt (cocolib/cocolib/common/
 * gsl_image.cpp:539-640): channels scaled by 1/255 on read (grey replicated to RGB, alpha dropped), written
 * as clamp(int(v * 255), 0, 255). rgb is 3 x h x w. Needs zlib at build time, else LFRV_E_IO. */
int lfrv_png_read(const char *path, int *w, int *h, float *rgb, size_t capacity);
int lfrv_png_write(const char *path, int w, int h, const float *rgb);

/* ---------------------------------------------------------------- synthetic light fields
 * No reference counterpart: the reference's datasets are absent, so seeded synthetic scenes stand in
 * for them. Pinhole cameras on an n x n grid (R = I, centres at baseline*(i-c, j-c, 0)), fronto-parallel
 * textured planes (each texture channel = 0.5 + 0.5/64 * sum of 64 seeded 2-D sinusoids), optional
 * Gaussian depth bumps, views rendered at ss x resolution and box-decimated, Gaussian sensor noise.
 */
typedef struct lfrv_scene_params {
    int      grid;            /* n for an n x n light field; the centre view is the target */
    int      w, h;            /* input view size */
    int      ss;              /* render supersampling of the inputs (box-decimated) */
    int      dsf;             /* target size = dsf * input size */
    double   baseline;
    int      nplanes;
    double   depths[16];      /* ascending; the last plane is a full background */
    int      nbumps;
    double   bump_amp;        /* world depth units */
    double   bump_sigma_px;   /* in target pixels */
    double   noise_sigma;
    double   focal_per_256;   /* target focal length per 256 target pixels of width (300) */
    uint64_t seed;
} lfrv_scene_params;

/* which: 1 = 3x3 256^2 (planes 1.0/1.5/2.5, baseline 0.05, noise 0.01);
 *        2 = 5x5 512^2 inputs rendered at 1024^2 and decimated, 5 planes + 20 bumps, baseline 0.03,
 *            noise 0.005, dsf 2. */
int lfrv_scene_params_preset(int which, lfrv_scene_params *p);
/* Sizes: views/depth V*3*h*w floats with V = grid^2 - 1; cams V+1 entries (inputs, then target);
 * gt 3*H*W floats. Any output pointer may be NULL. */
int lfrv_synth_scene(const lfrv_scene_params *p, float *views, float *depth, lfrv_camera *cams,
                     float *gt);
/* The same scene generated on the GPU into DEVICE buffers (context stream; returns when they are written), with
 * host cameras. It runs the same tracing code in double precision; the device's exp, log and cos may differ from
 * the host library's in the last bit, so views and depth maps equal lfrv_synth_scene's to the rounding of the final
 * float in all but rare pixels. For generating many scenes (training sets) at GPU speed. */
int lfrv_synth_scene_dev(lfrv_ctx *ctx, const lfrv_scene_params *p, float *d_views, float *d_depth,
                         lfrv_camera *cams, float *d_gt);

/* PSNR with peak 1.0 over all channels, excluding a border of `border` pixels
 * (gsl_image_psnr, cocolib/cocolib/common/gsl_image.cpp:991-1025 uses border 2). */
double lfrv_psnr(int W, int H, const float *a, const float *b, int border);

#ifdef __cplusplus
}
#endif

#endif /* LFRV_H */
