// lfrv_oracle.cpp -- CPU restatement of the reference's variational IBR hot path.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE. Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load this library, and only as the checker (or the timed CPU baseline). The product
// (liblfrv.so) never links, loads or calls it.
//
// Every function below restates one reference function and cites the file:line it follows
// (paths relative to the reference project root). The arithmetic is templated on the real type T:
//   T = double : the FP64 oracle every result's error is stated against;
//   T = float  : an FP32 mirror that follows the reference's float/double mixing, used to pin this
//                restatement against the reference's own kernels compiled on the CPU (oracle/_ref).
// Buffers are planar, channel-major, row-major, top-left origin, like the reference's device arrays.
//
// Pinning: the per-pixel kernels are checked bit-for-bit (float mirror) against the reference's kernel
// sources compiled for the CPU by oracle/build_ref.sh (see tests/test_oracle_ref.py); the reference has
// no golden vectors or fixtures for this path (its only regression tool, unitTest/, covers IBR_optical).
#include "lfrv.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace orc {

template <class T> using Vec = std::vector<T>;

static constexpr double kInvalidDepth = 1000.0;  // sources/openGL/frameBuffer.h:13

// ------------------------------------------------------------------ footprint of one source pixel
// cuda_set_A_bilinear, cocolib/cocolib/vtv/vtv_sr_kernels_unstructured.cu:658-718: the ks x ks weights
// (ks = dsf+1) of a dsf-wide box centred at tau-0.5, anchored at floor(px - dsf/2 + 1/2), normalised.
// Entries are stored at ks*i + j (i: row offset, j: column offset); the loop order (j outer, i inner)
// is the reference's and fixes the float summation order of the norm.
template <class T>
struct Footprint {
    int x0, y0, ks;
    T A[25];
    bool in[25];
};

template <class T>
inline void footprint(T tx, T ty, int dsf, int W, int H, Footprint<T> &fp) {
    const int ks = dsf + 1;
    fp.ks = ks;
    // px = warp_tau_x[m] - 0.5 is evaluated in double and stored in cuflt (vtv_sr_kernels_unstructured.cu:689)
    const T px = (T)((double)tx - 0.5);
    const T py = (T)((double)ty - 0.5);
    // (int)floor(px - cuflt(dsf)*0.5 + 0.5) is a double expression (:697)
    fp.x0 = (int)std::floor((double)px - (double)dsf * 0.5 + 0.5);
    fp.y0 = (int)std::floor((double)py - (double)dsf * 0.5 + 0.5);
    T norm = 0;
    for (int j = 0; j < ks; ++j) {
        for (int i = 0; i < ks; ++i) {
            const int x = fp.x0 + j, y = fp.y0 + i;
            const int e = ks * i + j;
            if (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1) {
                T dx = 1, dy = 1;
                if (j == 0) dx = (T)(((double)x + 0.5) - ((double)px - 0.5 * dsf));
                else if (j == ks - 1) dx = (T)(((double)px + 0.5 * dsf) - ((double)x - 0.5));
                if (i == 0) dy = (T)(((double)y + 0.5) - ((double)py - 0.5 * dsf));
                else if (i == ks - 1) dy = (T)(((double)py + 0.5 * dsf) - ((double)y - 0.5));
                fp.A[e] = dx * dy;
                fp.in[e] = true;
                norm += dx * dy;
            } else {
                fp.A[e] = 0;
                fp.in[e] = false;
            }
        }
    }
    if (norm != 0)
        for (int e = 0; e < ks * ks; ++e) fp.A[e] /= norm;
}

// Raw (un-normalised) dx*dy products, as setup_visibility_mask (sources/gradientIBR_kernels.cuh:4-55)
// evaluates them.
template <class T>
inline bool footprint_tap_nonzero(T tx, T ty, int dsf, int j, int i, int x, int y) {
    const int ks = dsf + 1;
    const T px = (T)((double)tx - 0.5), py = (T)((double)ty - 0.5);
    T dx = 1, dy = 1;
    if (j == 0) dx = (T)(((double)x + 0.5) - ((double)px - 0.5 * dsf));
    else if (j == ks - 1) dx = (T)(((double)px + 0.5 * dsf) - ((double)x - 0.5));
    if (i == 0) dy = (T)(((double)y + 0.5) - ((double)py - 0.5 * dsf));
    else if (i == ks - 1) dy = (T)(((double)py + 0.5 * dsf) - ((double)y - 0.5));
    return dx * dy != 0;
}

// Gather set of a view: cuda_convolution_nonsep_device_param tests tau_x<0 || tau_y<0 || tau_x>W || tau_y>H
// (vtv_sr_kernels_unstructured.cu:286).
template <class T>
inline bool in_gather(T tx, T ty, int W, int H) {
    return !(tx < 0 || ty < 0 || tx > W || ty > H);
}

// Splat set: the source pixels vtv_sr_init_forward_warp_structure_unstructured puts into cells
// (sources/optimization.cu:906-927): inside [0,W]x[0,H] and floor(tau-0.5) inside the target.
template <class T>
inline bool in_splat(T tx, T ty, int W, int H) {
    if (tx < 0 || ty < 0 || tx > W || ty > H) return false;
    const float uxv = (float)((double)tx - 0.5), uyv = (float)((double)ty - 0.5);
    const int px = (int)std::floor(uxv), py = (int)std::floor(uyv);
    return !(px < 0 || py < 0 || px > W - 1 || py > H - 1);
}

// ------------------------------------------------------------------ solver geometry per view
template <class T>
struct View {
    const T *img;   // 3 x n
    Vec<T> tx, ty;  // n
    Vec<T> dpx, dpy;  // sigma_z * dtau/dz (coco_vtv_sr_read_partial_tau, sources/optimization.cu:1208-1256)
    Vec<T> w;       // weights omega_i
    Vec<Footprint<T>> fp;
};

template <class T>
struct Problem {
    int w, h, W, H, dsf, V;
    Vec<View<T>> views;
};

template <class T>
void build_problem(Problem<T> &P, const lfrv_config &c, const T *views, const T *tau, int tau_ch,
                   const T *dpart) {
    P.w = c.w;
    P.h = c.h;
    P.dsf = c.dsf;
    P.W = c.w * c.dsf;
    P.H = c.h * c.dsf;
    P.V = c.nviews;
    const size_t n = (size_t)P.w * P.h;
    P.views.resize(P.V);
    for (int v = 0; v < P.V; ++v) {
        View<T> &vw = P.views[v];
        vw.img = views + (size_t)v * 3 * n;
        const T *tv = tau + (size_t)v * tau_ch * n;
        vw.tx.assign(tv, tv + n);
        vw.ty.assign(tv + n, tv + 2 * n);
        vw.dpx.resize(n);
        vw.dpy.resize(n);
        if (dpart) {
            const T *dp = dpart + (size_t)v * 3 * n;
            for (size_t m = 0; m < n; ++m) {
                vw.dpx[m] = dp[n + m] * dp[m];      // cuda_multiply_with_device(dpart_x, sigma_z)
                vw.dpy[m] = dp[2 * n + m] * dp[m];
            }
        }
        vw.w.assign(n, T(0));
        vw.fp.resize(n);
        for (size_t m = 0; m < n; ++m) footprint(vw.tx[m], vw.ty[m], P.dsf, P.W, P.H, vw.fp[m]);
    }
}

// v = A_i u  (cuda_convolution_nonsep_device_param, vtv_sr_kernels_unstructured.cu:268-363)
template <class T>
void gather(const Problem<T> &P, const View<T> &vw, int nch, const T *const *in, T *const *out) {
    const int n = P.w * P.h;
#pragma omp parallel for
    for (int m = 0; m < n; ++m) {
        for (int c = 0; c < nch; ++c) out[c][m] = 0;
        if (!in_gather(vw.tx[m], vw.ty[m], P.W, P.H)) continue;
        const Footprint<T> &fp = vw.fp[m];
        for (int j = 0; j < fp.ks; ++j)
            for (int i = 0; i < fp.ks; ++i) {
                const int x = fp.x0 + j, y = fp.y0 + i;
                if (0 <= x && x <= P.W - 1 && 0 <= y && y <= P.H - 1)
                    for (int c = 0; c < nch; ++c) out[c][m] += fp.A[fp.ks * i + j] * in[c][(size_t)y * P.W + x];
            }
    }
}

// O += A_i^T I, out_weight += A_i^T 1 (cuda_deconvolution_nonsep_device_param,
// vtv_sr_kernels_unstructured.cu:365-461) over the splat set. in_weights != nullptr gives the weighted
// variant (cuda_weighted_deconvolution_nonsep_device_param, :463-517). use_A=false splats weight 1.
template <class T>
void splat(const Problem<T> &P, const View<T> &vw, int nch, const T *const *in, T *const *out, T *out_weight,
           const T *in_weights, bool use_A = true) {
    const int n = P.w * P.h;
    for (int m = 0; m < n; ++m) {
        if (!in_splat(vw.tx[m], vw.ty[m], P.W, P.H)) continue;
        const Footprint<T> &fp = vw.fp[m];
        for (int j = 0; j < fp.ks; ++j)
            for (int i = 0; i < fp.ks; ++i) {
                const int x = fp.x0 + j, y = fp.y0 + i;
                if (!(0 <= x && x <= P.W - 1 && 0 <= y && y <= P.H - 1)) continue;
                const size_t o = (size_t)y * P.W + x;
                T weight = in_weights ? in_weights[m] : T(1);
                if (use_A) weight *= fp.A[fp.ks * i + j];
                if (out_weight) out_weight[o] += weight;
                for (int c = 0; c < nch; ++c) out[c][o] += weight * in[c][m];
            }
    }
}

// cuda_normalize_device (cocolib/cocolib/cuda/cuda_kernels.cu:322-339)
template <class T>
void normalize(size_t N, T *t, const T *wgt) {
    for (size_t o = 0; o < N; ++o)
        if (wgt[o] != 0) t[o] /= wgt[o];
}

// ------------------------------------------------------------------ Sobel of the luminance
// vtv_sr_compute_gradient_device, vtv_sr_kernels_unstructured.cu:96-148. Border pixels get 0; with a
// visibility mask, interior pixels whose 3x3 neighbourhood is not fully visible are NOT written.
// The luminance constants are double literals, so Y is a double expression rounded to cuflt.
template <class T>
inline T lum(T r, T g, T b) {
    return (T)(0.2126 * r + 0.7152 * g + 0.0722 * b);
}

template <class T>
void sobel(int W, int H, const T *r, const T *g, const T *b, T *gx, T *gy, const uint8_t *vis) {
#pragma omp parallel for
    for (int oy = 0; oy < H; ++oy)
        for (int ox = 0; ox < W; ++ox) {
            const size_t o = (size_t)oy * W + ox;
            T gX = 0, gY = 0;
            if (0 < ox && ox < W - 1 && 0 < oy && oy < H - 1) {
                const size_t ppo = (size_t)(oy - 1) * W + (ox - 1), pco = ppo + 1, pno = pco + 1;
                const size_t cpo = (size_t)oy * W + (ox - 1), cco = cpo + 1, cno = cco + 1;
                const size_t npo = (size_t)(oy + 1) * W + (ox - 1), nco = npo + 1, nno = nco + 1;
                if (vis && (!vis[ppo] || !vis[pco] || !vis[pno] || !vis[cpo] || !vis[cco] || !vis[cno] ||
                            !vis[npo] || !vis[nco] || !vis[nno]))
                    continue;
                const T Ypp = lum(r[ppo], g[ppo], b[ppo]), Ypc = lum(r[pco], g[pco], b[pco]);
                const T Ypn = lum(r[pno], g[pno], b[pno]), Ycp = lum(r[cpo], g[cpo], b[cpo]);
                const T Ycn = lum(r[cno], g[cno], b[cno]), Ynp = lum(r[npo], g[npo], b[npo]);
                const T Ync = lum(r[nco], g[nco], b[nco]), Ynn = lum(r[nno], g[nno], b[nno]);
                gX = (T)((Ypn + 2 * Ycn + Ynn - Ypp - 2 * Ycp - Ynp) / 8.);
                gY = (T)((Ynp + 2 * Ync + Ynn - Ypp - 2 * Ypc - Ypn) / 8.);
            }
            gx[o] = gX;
            gy[o] = gY;
        }
}

// ------------------------------------------------------------------ weights
// vtv_sr_angular_weights_device, vtv_sr_kernels_unstructured.cu:174-216
template <class T>
inline T angular_weight(T gx, T gy, T dpx, T dpy, T sigma, T thr) {
    const T norm = std::sqrt(gx * gx + gy * gy);
    if (norm > thr) {
        gx = gx / norm * thr;
        gy = gy / norm * thr;
    }
    T sg = gx * dpx + gy * dpy;
    if (sg > 0.5) sg = (T)0.5;
    return (T)(1.0 / (sg * sg + sigma * sigma));
}

// vtv_sr_gold_deform_weights_device, vtv_sr_kernels_unstructured.cu:218-266 (MAX_DEFORM_WEIGHT = 1)
template <class T>
inline T deform_weight(const T *tx, const T *ty, int m, int mx, int my, int w, int h, int W, int H) {
    auto out = [&](int k) { return tx[k] < 0 || tx[k] > W || ty[k] < 0 || ty[k] > H; };
    if (out(m)) return 0;
    if (mx == 0 || my == 0 || mx == w - 1 || my == h - 1) return 1;
    if (out(m - 1) || out(m + 1) || out(m - w) || out(m + w)) return 1;
    const T Dxx = (T)(0.5 * (tx[m + 1] - tx[m - 1]));
    const T Dyx = (T)(0.5 * (ty[m + 1] - ty[m - 1]));
    const T Dxy = (T)(0.5 * (tx[m + w] - tx[m - w]));
    const T Dyy = (T)(0.5 * (ty[m + w] - ty[m - w]));
    const T N = std::fabs(Dxx * Dyy - Dxy * Dyx);
    if (N > 1.0 / 1.0) return (T)(1.0 / N);
    return 1;
}

// Per-view weights from gradient buffers gx, gy (high res):
// the per-view part of coco_vtv_sr_compute_weights_unstructured, sources/optimization.cu:1094-1163.
template <class T>
void view_weights(const Problem<T> &P, View<T> &vw, const T *gx, const T *gy, T sigma, T thr) {
    const int n = P.w * P.h;
    Vec<T> wx(n), wy(n);
    const T *in[2] = {gx, gy};
    T *out[2] = {wx.data(), wy.data()};
    gather(P, vw, 2, in, out);
#pragma omp parallel for
    for (int m = 0; m < n; ++m) {
        const int mx = m % P.w, my = m / P.w;
        const T a = angular_weight(wx[m], wy[m], vw.dpx[m], vw.dpy[m], sigma, thr);
        const T d = deform_weight(vw.tx.data(), vw.ty.data(), m, mx, my, P.w, P.h, P.W, P.H);
        vw.w[m] = a * d;
    }
}

// ------------------------------------------------------------------ ROF inner iterations
// Dual step (coco_vtv_rof_dual_step_device, cocolib/cocolib/vtv/vtv_rof.cu:118-147), TV_F reprojection
// weighted by g (coco_vtv_rof_reproject_3D_tvf_weighted_device, vtv_rof.cu:280-320) and primal prox
// (cuda_rof_primal_prox_step_device, cocolib/cocolib/cuda/cuda_kernels.cu:504-532) applied to Uq in place,
// as vtv_sr_ista_step_unstructured calls them (sources/optimization.cu:1815-1828).
template <class T>
void rof_iterations(int W, int H, int niter, T tau, T sigma, T lam, const T *const F[3], const T *g,
                    T *const U[3], T *const PX[3], T *const PY[3]) {
    const size_t N = (size_t)W * H;
    for (int k = 0; k < niter; ++k) {
        for (int c = 0; c < 3; ++c) {
            const T *u = U[c];
            T *px = PX[c], *py = PY[c];
#pragma omp parallel for
            for (int oy = 0; oy < H; ++oy)
                for (int ox = 0; ox < W; ++ox) {
                    const size_t o = (size_t)oy * W + ox;
                    T grad = 0;
                    if (ox < W - 1) grad = u[o + 1] - u[o];
                    const T pxn = px[o] + sigma * grad;
                    grad = 0;
                    if (oy < H - 1) grad = u[o + W] - u[o];
                    const T pyn = py[o] + sigma * grad;
                    px[o] = pxn;
                    py[o] = pyn;
                }
        }
#pragma omp parallel for
        for (long long oo = 0; oo < (long long)N; ++oo) {
            const size_t o = (size_t)oo;
            const T a11 = PX[0][o], a21 = PX[1][o], a31 = PX[2][o];
            const T a12 = PY[0][o], a22 = PY[1][o], a32 = PY[2][o];
            T n = 0;
            n += (T)(std::pow(a11, (T)2) + std::pow(a21, (T)2) + std::pow(a31, (T)2));
            n += (T)(std::pow(a12, (T)2) + std::pow(a22, (T)2) + std::pow(a32, (T)2));
            n = std::sqrt(n);
            const T r = g[o];
            if (n > r) {
                n = r / n;
                PX[0][o] = a11 * n;
                PY[0][o] = a12 * n;
                PX[1][o] = a21 * n;
                PY[1][o] = a22 * n;
                PX[2][o] = a31 * n;
                PY[2][o] = a32 * n;
            }
        }
        for (int c = 0; c < 3; ++c) {
            T *u = U[c];
            const T *f = F[c], *px = PX[c], *py = PY[c];
#pragma omp parallel for
            for (int oy = 0; oy < H; ++oy)
                for (int ox = 0; ox < W; ++ox) {
                    const size_t o = (size_t)oy * W + ox;
                    T step = px[o] + py[o];
                    if (ox > 0) step -= px[o - 1];
                    if (oy > 0) step -= py[o - W];
                    const T unew = u[o] + tau * step;
                    u[o] = (tau * f[o] + lam * unew) / (tau + lam);
                }
        }
    }
}

// ------------------------------------------------------------------ separable Gaussian
// gsl_kernel_gauss_1xn (cocolib/cocolib/common/gsl_matrix_convolutions.cpp:42-63), copied to the device
// as float, applied by convolutionRowGPU / convolutionColumnGPU (cocolib/cocolib/cuda/
// cuda_convolutions.cu:110-238) with clamp-to-edge aprons: sum_k data[x+k] * kernel[R-k], k=-R..R.
template <class T>
void gaussian_blur(int W, int H, const T *in, T *out, int n = 11, double sigma = 2.0) {
    const int R = n / 2;
    std::vector<double> kd(n);
    double s = 0;
    for (int x = -R; x <= R; ++x) {
        kd[x + R] = std::exp(-0.5 * x * x / (sigma * sigma));
        s += kd[x + R];
    }
    std::vector<T> k(n);
    for (int i = 0; i < n; ++i) k[i] = (T)(float)(kd[i] / s);  // device kernel is float
    if (sizeof(T) == sizeof(double))
        for (int i = 0; i < n; ++i) k[i] = (T)(kd[i] / s);
    Vec<T> tmp((size_t)W * H);
#pragma omp parallel for
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            T sum = 0;
            for (int kk = -R; kk <= R; ++kk) {
                const int xx = std::min(std::max(x + kk, 0), W - 1);
                sum += in[(size_t)y * W + xx] * k[R - kk];
            }
            tmp[(size_t)y * W + x] = sum;
        }
#pragma omp parallel for
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            T sum = 0;
            for (int kk = -R; kk <= R; ++kk) {
                const int yy = std::min(std::max(y + kk, 0), H - 1);
                sum += tmp[(size_t)yy * W + x] * k[R - kk];
            }
            out[(size_t)y * W + x] = sum;
        }
}

// ------------------------------------------------------------------ push-pull hole filling
// reduce / expand, sources/optimization.cu:210-492 (float arrays in the reference).
template <class T>
void pp_reduce(int W, int H, int w, int h, const T *input, T *output) {
    const T a = (T)0.4f;
    const T kernel[5] = {(T)0.25f - (T)0.5f * a, (T)0.25f, a, (T)0.25f, (T)0.25f - (T)0.5f * a};
    Vec<T> tmp((size_t)W * std::max(h, 0));
    auto acc = [&](T &v, T &wt, T in, int k) {
        if (in != 0) {
            v += kernel[k] * in;
            wt += kernel[k];
        }
    };
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < W; ++j) {
            T v = 0, wt = 0;
            acc(v, wt, (2 * i - 2 < 0) ? input[j] : input[(size_t)(2 * i - 2) * W + j], 0);
            acc(v, wt, (2 * i - 1 < 0) ? input[j] : input[(size_t)(2 * i - 1) * W + j], 1);
            acc(v, wt, input[(size_t)(2 * i) * W + j], 2);
            acc(v, wt, (H - 1 < 2 * i + 1) ? input[(size_t)(H - 1) * W + j] : input[(size_t)(2 * i + 1) * W + j], 3);
            acc(v, wt, (H - 1 < 2 * i + 2) ? input[(size_t)(H - 1) * W + j] : input[(size_t)(2 * i + 2) * W + j], 4);
            tmp[(size_t)i * W + j] = (wt == 0) ? T(0) : v / wt;
        }
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < w; ++j) {
            const T *row = tmp.data() + (size_t)i * W;
            T v = 0, wt = 0;
            acc(v, wt, (2 * j - 2 < 0) ? row[0] : row[2 * j - 2], 0);
            acc(v, wt, (2 * j - 1 < 0) ? row[0] : row[2 * j - 1], 1);
            acc(v, wt, row[2 * j], 2);
            acc(v, wt, (W - 1 < 2 * j + 1) ? row[W - 1] : row[2 * j + 1], 3);
            acc(v, wt, (W - 1 < 2 * j + 2) ? row[W - 1] : row[2 * j + 2], 4);
            output[(size_t)i * w + j] = (wt == 0) ? T(0) : v / wt;
        }
}

inline void pp_reduce_bool(int W, int H, int w, int h, const uint8_t *input, uint8_t *output) {
    std::vector<uint8_t> tmp((size_t)W * std::max(h, 0));
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < W; ++j) {
            bool t = false;
            t = t || ((2 * i - 2 < 0) ? input[j] : input[(size_t)(2 * i - 2) * W + j]);
            t = t || ((2 * i - 1 < 0) ? input[j] : input[(size_t)(2 * i - 1) * W + j]);
            t = t || input[(size_t)(2 * i) * W + j];
            t = t || ((H - 1 < 2 * i + 1) ? input[(size_t)(H - 1) * W + j] : input[(size_t)(2 * i + 1) * W + j]);
            t = t || ((H - 1 < 2 * i + 2) ? input[(size_t)(H - 1) * W + j] : input[(size_t)(2 * i + 2) * W + j]);
            tmp[(size_t)i * W + j] = t;
        }
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < w; ++j) {
            const uint8_t *row = tmp.data() + (size_t)i * W;
            bool t = false;
            t = t || ((2 * j - 2 < 0) ? row[0] : row[2 * j - 2]);
            t = t || ((2 * j - 1 < 0) ? row[0] : row[2 * j - 1]);
            t = t || row[2 * j];
            t = t || ((W - 1 < 2 * j + 1) ? row[W - 1] : row[2 * j + 1]);
            t = t || ((W - 1 < 2 * j + 2) ? row[W - 1] : row[2 * j + 2]);
            output[(size_t)i * w + j] = t;
        }
}

// expand writes only the pixels of `output` that are not visible at that level (optimization.cu:430-492).
// A level of size 0 (the reference's fixed pyramid height 10 on images smaller than 2^10) holds no
// pixels; reading it is out of bounds in the reference. Here such reads yield 0.
template <class T>
void pp_expand(int W, int H, int w, int h, const T *input, T *output, const uint8_t *vis) {
    const T a = (T)0.4f;
    const T kernel[5] = {(T)0.25f - (T)0.5f * a, (T)0.25f, a, (T)0.25f, (T)0.25f - (T)0.5f * a};
    Vec<T> tmp((size_t)std::max(w, 0) * H);
    // Rows / columns past the coarser level (odd level sizes) clamp to its last row / column: the reference
    // reads beyond its array there (optimization.cu:447-452, 475-481).
    auto in_at = [&](int row, int col) -> T {
        return (w > 0 && h > 0) ? input[(size_t)std::min(row, h - 1) * w + std::min(col, w - 1)] : T(0);
    };
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < w; ++j) {
            T v = 0;
            if (i % 2 == 0) {
                v += 2 * kernel[0] * (((i - 2) / 2 < 0) ? in_at(0, j) : in_at((i - 2) / 2, j));
                v += 2 * kernel[2] * in_at(i / 2, j);
                v += 2 * kernel[4] * ((h - 1 < (i + 2) / 2) ? in_at(h - 1, j) : in_at((i + 2) / 2, j));
            } else {
                v += 2 * kernel[1] * (((i - 1) / 2 < 0) ? in_at(0, j) : in_at((i - 1) / 2, j));
                v += 2 * kernel[3] * ((h - 1 < (i + 1) / 2) ? in_at(h - 1, j) : in_at((i + 1) / 2, j));
            }
            tmp[(size_t)i * w + j] = v;
        }
    auto t_at = [&](int row, int col) -> T { return w > 0 ? tmp[(size_t)row * w + std::min(col, w - 1)] : T(0); };
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < W; ++j) {
            if (vis[(size_t)i * W + j]) continue;
            T v = 0;
            if (j % 2 == 0) {
                v += 2 * kernel[0] * (((j - 2) / 2 < 0) ? t_at(i, 0) : t_at(i, (j - 2) / 2));
                v += 2 * kernel[2] * t_at(i, j / 2);
                v += 2 * kernel[4] * ((w - 1 < (j + 2) / 2) ? t_at(i, w - 1) : t_at(i, (j + 2) / 2));
            } else {
                v += 2 * kernel[1] * (((j - 1) / 2 < 0) ? t_at(i, 0) : t_at(i, (j - 1) / 2));
                v += 2 * kernel[3] * ((w - 1 < (j + 1) / 2) ? t_at(i, w - 1) : t_at(i, (j + 1) / 2));
            }
            output[(size_t)i * W + j] = v;
        }
}

// coco_vtv_push_pull, sources/optimization.cu:544-651: pyramid height fixed to 10; the result written
// back is U = filled - U (cuda_subtract_from_device(temp, U), :643) when faithful, else U = filled.
template <class T>
void push_pull(int W, int H, const uint8_t *vis, T *U, bool faithful) {
    const int height = 10;
    for (int c = 0; c < 3; ++c) {
        T *u = U + (size_t)c * W * H;
        std::vector<Vec<T>> img(height + 1);
        std::vector<std::vector<uint8_t>> vp(height + 1);
        img[0].assign(u, u + (size_t)W * H);
        vp[0].assign(vis, vis + (size_t)W * H);
        auto dims = [&](int s, int &Ws, int &Hs, int &ws, int &hs) {
            Ws = (int)((unsigned)W / (unsigned)std::pow(2.0, (double)(s - 1)));
            Hs = (int)((unsigned)H / (unsigned)std::pow(2.0, (double)(s - 1)));
            ws = (int)((unsigned)W / (unsigned)std::pow(2.0, (double)s));
            hs = (int)((unsigned)H / (unsigned)std::pow(2.0, (double)s));
        };
        for (int s = 1; s <= height; ++s) {
            int Ws, Hs, ws, hs;
            dims(s, Ws, Hs, ws, hs);
            img[s].assign((size_t)ws * hs, T(0));
            vp[s].assign((size_t)ws * hs, 0);
            if (ws > 0 && hs > 0) {
                pp_reduce(Ws, Hs, ws, hs, img[s - 1].data(), img[s].data());
                pp_reduce_bool(Ws, Hs, ws, hs, vp[s - 1].data(), vp[s].data());
            }
        }
        for (int s = height; s > 0; --s) {
            int Ws, Hs, ws, hs;
            dims(s, Ws, Hs, ws, hs);
            if (Ws > 0 && Hs > 0) pp_expand(Ws, Hs, ws, hs, img[s].data(), img[s - 1].data(), vp[s - 1].data());
        }
        for (size_t o = 0; o < (size_t)W * H; ++o) u[o] = faithful ? (T)(img[0][o] - u[o]) : img[0][o];
    }
}

// ------------------------------------------------------------------ IBR_color state and stages
template <class T>
struct ColorState {
    Problem<T> P;
    lfrv_config cfg;
    size_t N;
    Vec<T> U[3], Uq[3], G[3], X1[3], X2[3], X1q, X2q, g, norm_mask, cov;
    Vec<T> gxs, gys;  // gradient buffers of the corrected mode (the reference writes into X1[0], X2[0])
    std::vector<uint8_t> vis;
    T alpha = 1;

    void init(const lfrv_config &c, const T *views, const T *tau, int tau_ch, const T *dpart) {
        cfg = c;
        build_problem(P, c, views, tau, tau_ch, dpart);
        N = (size_t)P.W * P.H;
        for (int i = 0; i < 3; ++i) {
            U[i].assign(N, 0);
            Uq[i].assign(N, 0);
            G[i].assign(N, 0);
            X1[i].assign(N, 0);
            X2[i].assign(N, 0);
        }
        X1q.assign(N, 0);
        X2q.assign(N, 0);
        gxs.assign(N, 0);
        gys.assign(N, 0);
        g.assign(N, 0);
        norm_mask.assign(N, 0);
        cov.assign(N, 0);
        vis.assign(N, 0);
    }
    const T *u(int c) const { return U[c].data(); }
};

// coco_vtv_sr_compute_weights_unstructured, sources/optimization.cu:1066-1167. The Sobel kernel writes
// into X1[0], X2[0] (the channel-0 dual variables) with the visibility mask (defect D5, faithful mode);
// the corrected mode writes into buffers of its own.
template <class T>
void color_compute_weights(ColorState<T> &S) {
    T *gx = S.cfg.faithful ? S.X1[0].data() : S.gxs.data();
    T *gy = S.cfg.faithful ? S.X2[0].data() : S.gys.data();
    sobel(S.P.W, S.P.H, S.U[0].data(), S.U[1].data(), S.U[2].data(), gx, gy, S.vis.data());
    for (auto &vw : S.P.views) view_weights(S.P, vw, gx, gy, (T)S.cfg.sigma_sensor, (T)S.cfg.ugrad_threshold);
}

// coco_vtv_setup_visibility_mask, sources/optimization.cu:33-135: coverage by splatting ones with A,
// visibility = coverage >= 1 (cuda_setup_visibility_mask_device, vtv_sr_kernels_unstructured.cu:76-94).
// The splat also accumulates into norm_mask, which is not cleared.
template <class T>
void color_visibility(ColorState<T> &S) {
    Vec<T> ones(S.N, T(1));
    std::fill(S.cov.begin(), S.cov.end(), T(0));
    for (auto &vw : S.P.views) {
        const T *in[1] = {ones.data()};
        T *out[1] = {S.cov.data()};
        splat(S.P, vw, 1, in, out, S.norm_mask.data(), (const T *)nullptr);
    }
    for (size_t o = 0; o < S.N; ++o) S.vis[o] = S.cov[o] < 1.0 ? 0 : 1;
}

// Weighted average of the splatted views (coco_vtv_sr_compute_initial_image, sources/optimization.cu:
// 1300-1350) then push-pull (:1357).
template <class T>
void color_initial_image(ColorState<T> &S, bool fill) {
    for (int c = 0; c < 3; ++c) std::fill(S.U[c].begin(), S.U[c].end(), T(0));
    std::fill(S.norm_mask.begin(), S.norm_mask.end(), T(0));
    const size_t n = (size_t)S.P.w * S.P.h;
    for (auto &vw : S.P.views) {
        const T *in[3] = {vw.img, vw.img + n, vw.img + 2 * n};
        T *out[3] = {S.U[0].data(), S.U[1].data(), S.U[2].data()};
        splat(S.P, vw, 3, in, out, S.norm_mask.data(), vw.w.data());
    }
    for (int c = 0; c < 3; ++c) normalize(S.N, S.U[c].data(), S.norm_mask.data());
    if (fill) {
        Vec<T> all(3 * S.N);
        for (int c = 0; c < 3; ++c) std::copy(S.U[c].begin(), S.U[c].end(), all.begin() + c * S.N);
        push_pull(S.P.W, S.P.H, S.vis.data(), all.data(), S.cfg.faithful != 0);
        for (int c = 0; c < 3; ++c) std::copy(all.begin() + c * S.N, all.begin() + (c + 1) * S.N, S.U[c].begin());
    }
}

// coco_vtv_sr_init_regularizer_weight_unstructured, sources/optimization.cu:2251-2338 with
// vtv_sr_init_regularizer_weight_device (cocolib/cocolib/vtv/vtv_sr_kernels.cu:1172-1195).
template <class T>
void color_regularizer(ColorState<T> &S) {
    // The reference never clears the coverage accumulator here (defect D6, faithful mode).
    if (!S.cfg.faithful) std::fill(S.norm_mask.begin(), S.norm_mask.end(), T(0));
    Vec<T> m(S.N, T(0));
    for (auto &vw : S.P.views) {
        const T *in[1] = {vw.w.data()};
        T *out[1] = {m.data()};
        splat(S.P, vw, 1, in, out, S.norm_mask.data(), (const T *)nullptr);
    }
    normalize(S.N, m.data(), S.norm_mask.data());
    const T s2 = (T)S.cfg.sigma_sensor * (T)S.cfg.sigma_sensor;
    for (size_t o = 0; o < S.N; ++o) m[o] *= s2;
    const T lmax = (T)S.cfg.lambda_max_factor * (T)S.cfg.lambda, lmin = (T)S.cfg.lambda;
    const T mmax = (T)S.P.V;
    Vec<T> g0(S.N);
    for (size_t o = 0; o < S.N; ++o) g0[o] = (m[o] == 0) ? lmax : std::max(lmin, lmax - m[o] / mmax);
    gaussian_blur(S.P.W, S.P.H, g0.data(), S.g.data());
}

// Reference energy, coco_vtv_sr_primal_energy_unstructured, sources/optimization.cu:1477-1717.
// Host sums are float accumulations in the reference (cuflt); here they are T accumulations.
template <class T>
T color_energy(ColorState<T> &S, T *e_tv_out = nullptr, T *e_data_out = nullptr) {
    sobel(S.P.W, S.P.H, S.U[0].data(), S.U[1].data(), S.U[2].data(), S.X1q.data(), S.X2q.data(), S.vis.data());
    T e_tv = 0;
    for (size_t i = 0; i < S.N; ++i) e_tv += std::abs(S.X1q[i]);
    for (size_t i = 0; i < S.N; ++i) e_tv += std::abs(S.X2q[i]);
    const size_t n = (size_t)S.P.w * S.P.h;
    Vec<T> tmp(n, T(0));
    Vec<T> v0(n), v1(n), v2(n);
    const T s2 = (T)S.cfg.sigma_sensor * (T)S.cfg.sigma_sensor;
    for (auto &vw : S.P.views) {
        const T *in[3] = {S.U[0].data(), S.U[1].data(), S.U[2].data()};
        T *out[3] = {v0.data(), v1.data(), v2.data()};
        gather(S.P, vw, 3, in, out);
        for (int c = 0; c < 3; ++c) {
            T *vc = out[c];
            const T *img = vw.img + c * n;
            for (size_t m = 0; m < n; ++m) {
                T d = vc[m] - img[m];
                d = d * d;
                d = d * vw.w[m];
                d = d * s2;
                tmp[m] += d;
            }
        }
    }
    T e_int = 0;
    for (size_t m = 0; m < n; ++m) e_int += tmp[m];
    // The gradient data term (dt_beta) is multiplied by dt_beta; it is evaluated only when dt_beta != 0.
    T e_grad = 0;
    if (S.cfg.dt_beta != 0) {
        Vec<T> ugx(S.N), ugy(S.N), vgx(n), vgy(n), agx(n), agy(n);
        std::fill(tmp.begin(), tmp.end(), T(0));
        for (auto &vw : S.P.views) {
            sobel(S.P.W, S.P.H, S.U[0].data(), S.U[1].data(), S.U[2].data(), ugx.data(), ugy.data(), (const uint8_t *)nullptr);
            sobel(S.P.w, S.P.h, vw.img, vw.img + n, vw.img + 2 * n, vgx.data(), vgy.data(), (const uint8_t *)nullptr);
            const T *in[2] = {ugx.data(), ugy.data()};
            T *out[2] = {agx.data(), agy.data()};
            gather(S.P, vw, 2, in, out);
            for (size_t m = 0; m < n; ++m) {
                T a = agx[m] - vgx[m], b = agy[m] - vgy[m];
                a = (T)std::pow(a, (T)2);
                b = (T)std::pow(b, (T)2);
                if (S.cfg.gw_type != 0) {
                    a *= vw.w[m];
                    b *= vw.w[m];
                    a *= s2;
                    b *= s2;
                }
                tmp[m] += a;
                tmp[m] += b;
            }
        }
        for (size_t m = 0; m < n; ++m) e_grad += tmp[m];
    }
    if (e_tv_out) *e_tv_out = e_tv;
    if (e_data_out) *e_data_out = e_int;
    return (T)S.cfg.lambda * e_tv + (T)S.cfg.dt_alpha * e_int + (T)S.cfg.dt_beta * e_grad;
}

// vtv_sr_dataterm_intensities, sources/optimization.cu:1835-1966: G += alpha * sigma^2 *
// normalise(sum_i A_i^T [w_i (A_i U - v_i)]). norm_mask is cleared and re-accumulated.
template <class T>
void color_dataterm(ColorState<T> &S, T *Gint[3]) {
    const size_t n = (size_t)S.P.w * S.P.h;
    for (int c = 0; c < 3; ++c) std::fill(Gint[c], Gint[c] + S.N, T(0));
    std::fill(S.norm_mask.begin(), S.norm_mask.end(), T(0));
    Vec<T> t0(n), t1(n), t2(n);
    for (auto &vw : S.P.views) {
        const T *in[3] = {S.U[0].data(), S.U[1].data(), S.U[2].data()};
        T *out[3] = {t0.data(), t1.data(), t2.data()};
        gather(S.P, vw, 3, in, out);
        for (int c = 0; c < 3; ++c) {
            const T *img = vw.img + c * n;
            for (size_t m = 0; m < n; ++m) out[c][m] -= img[m];
        }
        for (int c = 0; c < 3; ++c)
            for (size_t m = 0; m < n; ++m) out[c][m] *= vw.w[m];
        const T *sin_[3] = {t0.data(), t1.data(), t2.data()};
        splat(S.P, vw, 3, sin_, Gint, S.norm_mask.data(), (const T *)nullptr);
    }
    for (int c = 0; c < 3; ++c) normalize(S.N, Gint[c], S.norm_mask.data());
    const T s2 = (T)S.cfg.sigma_sensor * (T)S.cfg.sigma_sensor;
    for (int c = 0; c < 3; ++c)
        for (size_t o = 0; o < S.N; ++o) {
            Gint[c][o] *= s2;
            S.G[c][o] += (T)S.cfg.dt_alpha * Gint[c][o];
        }
}

// cuda_laplacian_device (cocolib/cocolib/vtv/vtv_sr_kernels_unstructured.cu:720-760) without a visibility
// mask: the mean of the in-image 4-neighbours (summed left, up, right, down) minus the centre.
template <class T>
void laplacian(int W, int H, const T *in, T *out) {
    for (int oy = 0; oy < H; ++oy)
        for (int ox = 0; ox < W; ++ox) {
            const size_t o = (size_t)oy * W + ox;
            T v = 0, wt = 0;
            if (ox > 0) { v += in[o - 1]; wt += 1; }
            if (oy > 0) { v += in[o - W]; wt += 1; }
            if (ox < W - 1) { v += in[o + 1]; wt += 1; }
            if (oy < H - 1) { v += in[o + W]; wt += 1; }
            v /= wt;
            v -= in[o];
            out[o] = v;
        }
}

// vtv_sr_dataterm_gradients, sources/optimization.cu:1969-2116 (dt_beta > 0): per view the residual
// dsf^2 A_i lap(U) - lap(v_i) (times omega_i when gw_type != 0) is splatted with A_i^T; the sum is normalised
// by the splatted coverage, scaled by sigma^2 (gw_type != 0) and by -gradient_step, and added as
// G += dt_beta * G_gradients. norm_mask is cleared and re-accumulated (the same coverage as the intensities).
template <class T>
void color_dataterm_gradients(ColorState<T> &S) {
    const size_t n = (size_t)S.P.w * S.P.h, N = S.N;
    Vec<T> gg[3] = {Vec<T>(N, T(0)), Vec<T>(N, T(0)), Vec<T>(N, T(0))};
    std::fill(S.norm_mask.begin(), S.norm_mask.end(), T(0));
    Vec<T> lu[3] = {Vec<T>(N), Vec<T>(N), Vec<T>(N)};
    for (int c = 0; c < 3; ++c) laplacian(S.P.W, S.P.H, S.U[c].data(), lu[c].data());
    Vec<T> t0(n), t1(n), t2(n), lv(n);
    const T dsf2 = (T)(float)(S.P.dsf * S.P.dsf);
    for (auto &vw : S.P.views) {
        const T *in[3] = {lu[0].data(), lu[1].data(), lu[2].data()};
        T *out[3] = {t0.data(), t1.data(), t2.data()};
        gather(S.P, vw, 3, in, out);
        for (int c = 0; c < 3; ++c) {
            for (size_t m = 0; m < n; ++m) out[c][m] *= dsf2;
            laplacian(S.P.w, S.P.h, vw.img + c * n, lv.data());
            for (size_t m = 0; m < n; ++m) out[c][m] -= lv[m];
        }
        if (S.cfg.gw_type != 0)
            for (int c = 0; c < 3; ++c)
                for (size_t m = 0; m < n; ++m) out[c][m] *= vw.w[m];
        const T *sin_[3] = {t0.data(), t1.data(), t2.data()};
        T *gp[3] = {gg[0].data(), gg[1].data(), gg[2].data()};
        splat(S.P, vw, 3, sin_, gp, S.norm_mask.data(), (const T *)nullptr);
    }
    const T s2 = (T)S.cfg.sigma_sensor * (T)S.cfg.sigma_sensor;
    const T step = -(T)S.cfg.gradient_step;
    for (int c = 0; c < 3; ++c) {
        normalize(N, gg[c].data(), S.norm_mask.data());
        for (size_t o = 0; o < N; ++o) {
            T v = gg[c][o];
            if (S.cfg.gw_type != 0) v *= s2;
            v *= step;
            S.G[c][o] += (T)S.cfg.dt_beta * v;
        }
    }
}

// The primal-dual constants set by coco_vtv_sr_iteration_fista_unstructured (sources/optimization.cu:
// 1736-1748): tau = sigma = 0.3/sqrt(8), L = 1/lambda; the F scale is -1/(lambda*L) computed in float.
template <class T>
struct RofConsts {
    T tau, sigma, lam_prox, fscale;
};
template <class T>
RofConsts<T> rof_consts(const lfrv_config &c) {
    RofConsts<T> k;
    k.tau = (T)(0.3 / std::sqrt(8.0));
    k.sigma = (T)(0.3 / std::sqrt(8.0));
    if (sizeof(T) == sizeof(float)) {
        const float L = (float)(1.0 / c.lambda);
        k.lam_prox = (T)(float)(1.0 / L);
        k.fscale = (T)(float)(-1.0 / (double)(c.lambda * L));
    } else {
        k.lam_prox = (T)c.lambda;
        k.fscale = (T)-1.0;
    }
    return k;
}

// One FISTA iteration (coco_vtv_sr_iteration_fista_unstructured, sources/optimization.cu:1736-1748;
// vtv_sr_ista_step_unstructured :1751-1832; coco_vtv_rof_overrelaxation vtv_rof.cu:28-56).
template <class T>
void color_fista_iteration(ColorState<T> &S) {
    const size_t N = S.N;
    for (int c = 0; c < 3; ++c) {
        S.Uq[c] = S.U[c];
        std::fill(S.G[c].begin(), S.G[c].end(), T(0));
    }
    if (S.cfg.dt_alpha > 0) {
        Vec<T> gi[3] = {Vec<T>(N), Vec<T>(N), Vec<T>(N)};
        T *gp[3] = {gi[0].data(), gi[1].data(), gi[2].data()};
        color_dataterm(S, gp);
    }
    if (S.cfg.dt_beta > 0) color_dataterm_gradients(S);
    const RofConsts<T> k = rof_consts<T>(S.cfg);
    for (int c = 0; c < 3; ++c)
        for (size_t o = 0; o < N; ++o) {
            T gv = std::min((T)1.0f, std::max((T)-1.0f, S.G[c][o]));
            gv *= k.fscale;
            gv += S.Uq[c][o];
            S.G[c][o] = std::min((T)1.0f, std::max((T)0.0f, gv));
        }
    const T *F[3] = {S.G[0].data(), S.G[1].data(), S.G[2].data()};
    T *U[3] = {S.Uq[0].data(), S.Uq[1].data(), S.Uq[2].data()};
    T *PX[3] = {S.X1[0].data(), S.X1[1].data(), S.X1[2].data()};
    T *PY[3] = {S.X2[0].data(), S.X2[1].data(), S.X2[2].data()};
    rof_iterations(S.P.W, S.P.H, S.cfg.niter, k.tau, k.sigma, k.lam_prox, F, S.g.data(), U, PX, PY);
    const T alpha_new = (T)(0.5 * (1.0 + std::sqrt(1.0 + 4.0 * std::pow((double)S.alpha, 2.0))));
    const T theta = (T)(((double)S.alpha - 1.0) / (double)alpha_new);
    for (int c = 0; c < 3; ++c)
        for (size_t o = 0; o < N; ++o) {
            const T uv = S.U[c][o], uqv = S.Uq[c][o];
            S.Uq[c][o] = uv + theta * (uqv - uv);
            S.U[c][o] = uqv;
        }
    S.alpha = alpha_new;
}

// ------------------------------------------------------------------ IBR_color, corrected mode
// No reference counterpart: the objective the reference's ISTA step (sources/optimization.cu:1751-1832) aims at,
// solved to a certified primal-dual gap.
//   E(u) = f(u) + lambda J_g(u) over the box [0, 1]^{3N},
//   f(u) = alpha sigma^2 / 2 sum_i sum_{m in S_i} w_im |A_i u - v_i|^2_m   (S_i: the splat set of view i, the same
//          set the data term's gradient splats over, so that grad f = alpha sigma^2 sum_i A_i^T w_i (A_i u - v_i)),
//   J_g(u) = sum_x g_x |grad u(x)|_F (forward differences with zero at the last column / row, Frobenius norm over
//          the 3 channels and 2 directions: the weighted TV_F whose dual ball vtv_rof.cu:280-320 projects onto).
// Solver: FISTA in the diagonal metric D = max(alpha sigma^2 sum_i A_i^T w_i, kTvDelta), which majorises the
// Hessian of f (rows of A_i sum to 1, so by Cauchy-Schwarz (A_i u)^2 <= A_i (u^2)), with the momentum restarted
// whenever the energy rises (function-value restart, O'Donoghue and Candes 2015). Each step is the weighted ROF
// problem min_u lambda J_g(u) + 1/2 |u - F|^2_D over the box with F = y - grad f(y) / D, solved by kTvInner
// iterations of the fast gradient projection on its dual (|p(x)| <= g_x), warm-started from the last dual.
// Certificate: for |p| <= g and u in the box, with c = grad f(u) - lambda div p,
//   E(u) - E* <= gap(u, p) = lambda sum_x [g_x |grad u(x)|_F - <grad u(x), p(x)>] + sum [u c - min(0, c)],
// (the Fenchel dual of the problem with the data term's dual variable at its optimum for u). The solver stops
// when gap / E <= cfg.cg_gap_tol or after cfg.niter outer iterations.
constexpr int kTvInner = 200;
// The dual field p and its momentum point are double in both builds: in float, their rounding (a few ulp of
// |p| <= g) leaves lambda div p, and with it the certificate's box term, a noise floor near 4e-4 relative at 256^2.
// The GPU stores the dual in FP64 too (its arithmetic FP32 far from the floor, double-float near it) with FP32
// iterates, so the FP32 mirror stays its like-for-like reference.
using TvDual = double;
constexpr double kTvDelta = 1.0;

// grad f(u) (3 planes) and f(u): residuals over the splat set.
template <class T>
double tv_grad_f(const ColorState<T> &S, const Vec<T> *U, Vec<T> *gf) {
    const size_t n = (size_t)S.P.w * S.P.h, N = S.N;
    const double as2 = (double)S.cfg.dt_alpha * (double)S.cfg.sigma_sensor * (double)S.cfg.sigma_sensor;
    for (int c = 0; c < 3; ++c) std::fill(gf[c].begin(), gf[c].end(), T(0));
    double f = 0;
    Vec<T> r0(n), r1(n), r2(n);
    for (const auto &vw : S.P.views) {
        T *r[3] = {r0.data(), r1.data(), r2.data()};
#pragma omp parallel for reduction(+ : f)
        for (long long mm = 0; mm < (long long)n; ++mm) {
            const size_t m = (size_t)mm;
            for (int c = 0; c < 3; ++c) r[c][m] = 0;
            if (!in_splat(vw.tx[m], vw.ty[m], S.P.W, S.P.H)) continue;
            const Footprint<T> &fp = vw.fp[m];
            T a[3] = {0, 0, 0};
            for (int j = 0; j < fp.ks; ++j)
                for (int i = 0; i < fp.ks; ++i) {
                    const int x = fp.x0 + j, y = fp.y0 + i;
                    if (0 <= x && x <= S.P.W - 1 && 0 <= y && y <= S.P.H - 1)
                        for (int c = 0; c < 3; ++c) a[c] += fp.A[fp.ks * i + j] * U[c][(size_t)y * S.P.W + x];
                }
            for (int c = 0; c < 3; ++c) {
                const T d = a[c] - vw.img[c * n + m];
                f += 0.5 * as2 * (double)vw.w[m] * (double)d * (double)d;
                r[c][m] = vw.w[m] * d;
            }
        }
        const T *in[3] = {r0.data(), r1.data(), r2.data()};
        T *out[3] = {gf[0].data(), gf[1].data(), gf[2].data()};
        splat(S.P, vw, 3, in, out, (T *)nullptr, (const T *)nullptr);
    }
    for (int c = 0; c < 3; ++c)
        for (size_t o = 0; o < N; ++o) gf[c][o] = (T)(as2 * (double)gf[c][o]);
    return f;
}

// div of a dual field (the negative adjoint of the forward gradient with zero at the last column / row).
template <class T>
inline T tv_div_at(const T *px, const T *py, int W, int H, int x, int y) {
    const size_t o = (size_t)y * W + x;
    T d = 0;
    if (x < W - 1) d += px[o];
    if (x > 0) d -= px[o - 1];
    if (y < H - 1) d += py[o];
    if (y > 0) d -= py[o - W];
    return d;
}

// kTvInner iterations of FGP on the dual of min_u J_g(u) + sum_x (1 / (2 lam_x)) |u(x) - F(x)|^2 over the box,
// lam_x = lambda / D_x: u(q) = clamp(F + lam div q, 0, 1), p <- proj_{|.| <= g}(q + grad u(q) / L_x),
// q <- p + (s - 1) / s' (p - p_old). The step is per pixel: the dual's Hessian grad diag(lam) grad^T is at most
// diag(L) with L_x = 8 max(lam_x, lam_{x+1}, lam_{x+W}) (each dual entry enters the divergence at two pixels, each
// divergence has four terms), so the fast gradient projection converges in that metric; the ball projection stays
// a radial scaling since L_x is one scalar for the six entries of pixel x. P: px (3 planes), py (3 planes).
template <class T, class TP>
void tv_fgp(int W, int H, const Vec<T> *F, const Vec<T> &lam, const Vec<T> &g, const Vec<T> &Linv, Vec<TP> *P,
            int iters, Vec<T> *U) {
    const size_t N = (size_t)W * H;
    Vec<TP> Q[6], Pn[6];
    Vec<T> u[3];
    for (int k = 0; k < 6; ++k) Q[k] = P[k], Pn[k].assign(N, 0);
    for (int c = 0; c < 3; ++c) u[c].assign(N, 0);
    double s = 1;
    auto primal = [&](const Vec<TP> *q, Vec<T> *out) {
        for (int c = 0; c < 3; ++c) {
#pragma omp parallel for
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x) {
                    const size_t o = (size_t)y * W + x;
                    const T v = F[c][o] + lam[o] * (T)tv_div_at(q[c].data(), q[3 + c].data(), W, H, x, y);
                    out[c][o] = std::min((T)1, std::max((T)0, v));
                }
        }
    };
    for (int it = 0; it < iters; ++it) {
        primal(Q, u);
        const double s1 = 0.5 * (1.0 + std::sqrt(1.0 + 4.0 * s * s));
        const TP beta = (TP)((s - 1.0) / s1);
#pragma omp parallel for
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t o = (size_t)y * W + x;
                TP v[6];
                TP nrm = 0;
                for (int c = 0; c < 3; ++c) {
                    const T gxv = x < W - 1 ? u[c][o + 1] - u[c][o] : T(0);
                    const T gyv = y < H - 1 ? u[c][o + W] - u[c][o] : T(0);
                    v[c] = Q[c][o] + (TP)(gxv * Linv[o]);
                    v[3 + c] = Q[3 + c][o] + (TP)(gyv * Linv[o]);
                    nrm += v[c] * v[c] + v[3 + c] * v[3 + c];
                }
                nrm = std::sqrt(nrm);
                const TP sc = nrm > (TP)g[o] ? (TP)g[o] / nrm : TP(1);
                for (int k = 0; k < 6; ++k) {
                    const TP pn = v[k] * sc;
                    Q[k][o] = pn + beta * (pn - P[k][o]);
                    Pn[k][o] = pn;
                }
            }
        for (int k = 0; k < 6; ++k) std::swap(P[k], Pn[k]);
        s = s1;
    }
    primal(P, U);
}

// E(u) and the certified gap for the dual p (see above); J_g(u) through *J.
template <class T, class TP>
double tv_gap(int W, int H, const Vec<T> *U, const Vec<T> *gf, const Vec<TP> *P, const Vec<T> &g, double lambda,
              double *J) {
    double tv = 0, inner = 0, box = 0;
#pragma omp parallel for reduction(+ : tv, inner, box)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * W + x;
            double n2 = 0;
            for (int c = 0; c < 3; ++c) {
                const double gxv = x < W - 1 ? (double)U[c][o + 1] - (double)U[c][o] : 0.0;
                const double gyv = y < H - 1 ? (double)U[c][o + W] - (double)U[c][o] : 0.0;
                n2 += gxv * gxv + gyv * gyv;
                inner += gxv * (double)P[c][o] + gyv * (double)P[3 + c][o];
                const double cc =
                    (double)gf[c][o] - lambda * (double)tv_div_at(P[c].data(), P[3 + c].data(), W, H, x, y);
                box += (double)U[c][o] * cc - std::min(0.0, cc);
            }
            tv += (double)g[o] * std::sqrt(n2);
        }
    *J = tv;
    return lambda * (tv - inner) + box;
}

// One meta iteration of the corrected IBR_color solve on S.U (weights and g already set). Returns the outer
// iterations run; *E_out, *gap_out: energy and relative gap of the returned iterate. trace: E after each outer
// iteration (and of the start), at most trace_cap entries from trace_pos on.
template <class T>
int tv_solve(ColorState<T> &S, int max_outer, double tol, double *E_out, double *gap_out, double *trace,
             int trace_cap, int *trace_pos, const Vec<T> *P0 = nullptr) {
    const int W = S.P.W, H = S.P.H;
    const size_t N = S.N;
    const double lambda = (double)S.cfg.lambda;
    const double as2 = (double)S.cfg.dt_alpha * (double)S.cfg.sigma_sensor * (double)S.cfg.sigma_sensor;
    // metric D and the per-pixel prox parameter lambda / D
    Vec<T> Dm(N, T(0)), lam(N);
    for (const auto &vw : S.P.views) {
        const T *in[1] = {vw.w.data()};
        T *out[1] = {Dm.data()};
        splat(S.P, vw, 1, in, out, (T *)nullptr, (const T *)nullptr);
    }
    for (size_t o = 0; o < N; ++o) {
        Dm[o] = (T)std::max(as2 * (double)Dm[o], kTvDelta);
        lam[o] = (T)(lambda / (double)Dm[o]);
    }
    Vec<T> Linv(N);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * W + x;
            T m = lam[o];
            if (x < W - 1) m = std::max(m, lam[o + 1]);
            if (y < H - 1) m = std::max(m, lam[o + W]);
            Linv[o] = (T)(1.0 / (8.0 * (double)m));
        }
    Vec<T> u[3], up[3], gf[3], gfp[3], Fy[3];
    Vec<TvDual> P[6];
    for (int c = 0; c < 3; ++c) {
        u[c].resize(N);
        for (size_t o = 0; o < N; ++o) u[c][o] = std::min((T)1, std::max((T)0, S.U[c][o]));
        up[c] = u[c];
        gf[c].assign(N, 0);
        gfp[c].assign(N, 0);
        Fy[c].assign(N, 0);
    }
    for (int k = 0; k < 6; ++k) P[k].assign(N, TvDual(0));
    double t = 1.0, E = 0, gap = 1e300, E_prev = 1e300;
    int k;
    for (k = 0;; ++k) {
        const double f = tv_grad_f(S, u, gf);
        double J = 0;
        const double g_abs = tv_gap(W, H, u, gf, P, S.g, lambda, &J);
        E = f + lambda * J;
        gap = E > 0 ? g_abs / E : 1e300;
        if (trace && *trace_pos < trace_cap) trace[(*trace_pos)++] = E;
        if (k >= max_outer || (tol > 0 && gap <= tol)) break;
        if (E > E_prev) t = 1.0;  // function-value restart of the momentum (O'Donoghue and Candes)
        E_prev = E;
        // FISTA step: y = u + theta (u - u_prev); grad f(y) = (1 + theta) grad f(u) - theta grad f(u_prev)
        const double t1 = 0.5 * (1.0 + std::sqrt(1.0 + 4.0 * t * t));
        const double theta = k == 0 ? 0.0 : (t - 1.0) / t1;
        for (int c = 0; c < 3; ++c)
            for (size_t o = 0; o < N; ++o) {
                const double y = (double)u[c][o] + theta * ((double)u[c][o] - (double)up[c][o]);
                const double gy = (1.0 + theta) * (double)gf[c][o] - theta * (double)gfp[c][o];
                Fy[c][o] = (T)(y - gy / (double)Dm[o]);
            }
        t = t1;
        for (int c = 0; c < 3; ++c) {
            std::swap(up[c], u[c]);
            std::swap(gfp[c], gf[c]);
        }
        tv_fgp(W, H, Fy, lam, S.g, Linv, P, kTvInner, u);
    }
    for (int c = 0; c < 3; ++c) S.U[c] = u[c];
    *E_out = E;
    *gap_out = gap;
    return k;
}

// sr_compare_images, sources/super-resolution.cpp:16-51
template <class T>
int moving_pixels(const ColorState<T> &S, const Vec<T> prev[3]) {
    int nM = 0;
    for (size_t o = 0; o < S.N; ++o) {
        double mx = 0;
        for (int c = 0; c < 3; ++c) mx = std::max(mx, std::fabs((double)S.U[c][o] - (double)prev[c][o]));
        if (!(mx < (double)(float)1e-3)) ++nM;  // MAX_DIFF_THRESHOLD is a cuflt (super-resolution.cpp:178)
    }
    return nM;
}

// sr_synthesize_view, sources/super-resolution.cpp:54-338.
template <class T>
void ibr_color(const lfrv_config &cfg, const T *views, const T *tau, int tau_ch, const T *dpart, const T *init,
               T *out, lfrv_stats *st) {
    ColorState<T> S;
    S.init(cfg, views, tau, tau_ch, dpart);
    if (st) st->trace_length = 0;
    color_compute_weights(S);   // super-resolution.cpp:157 (U = 0, visibility all false)
    color_visibility(S);        // :160
    if (init) {
        for (int c = 0; c < 3; ++c) std::copy(init + c * S.N, init + (c + 1) * S.N, S.U[c].begin());
    } else {
        color_initial_image(S, true);  // :165
    }
    Vec<T> prev_meta[3], prev[3];
    for (int c = 0; c < 3; ++c) prev_meta[c] = prev[c] = S.U[c];
    // EPSILON_TOL, PERCENT_MOVING are cuflt constants (super-resolution.cpp:177-179)
    const double EPS = (double)(float)1e-4;
    const float PERCENT_MOVING = (float)0.01;
    T energy = 0, previous_energy = 0, previous_energy_reweight = 0;
    int r, total_k = 0, reason = 0;
    double tv_gap_last = 0;
    int trace_pos = 0;
    const bool traced = st && st->energy_trace && st->trace_capacity > 0;
    for (r = 0; r < cfg.nmeta_iter; ++r) {
        color_compute_weights(S);
        color_regularizer(S);
        if (!cfg.faithful) {  // corrected mode: the true objective to a certified gap
            double Ec = 0;
            total_k += tv_solve(S, cfg.niter, cfg.cg_gap_tol, &Ec, &tv_gap_last, traced ? st->energy_trace : nullptr,
                                traced ? st->trace_capacity : 0, &trace_pos);
            energy = (T)Ec;
            reason = (cfg.cg_gap_tol > 0 && tv_gap_last <= cfg.cg_gap_tol) ? 4 : 0;
            if (traced) st->trace_length = trace_pos;
            continue;
        }
        energy = color_energy(S);
        previous_energy = energy;
        int k;
        for (k = 0; k < cfg.niter; ++k) {
            color_fista_iteration(S);
            ++total_k;
            energy = color_energy(S);
            if (st && st->energy_trace && total_k - 1 < st->trace_capacity) {
                st->energy_trace[total_k - 1] = (double)energy;
                st->trace_length = total_k;
            }
            if (!cfg.early_exit) continue;
            if ((double)energy < EPS) {
                reason = 1;
                break;
            }
            const double rel = std::fabs((double)((energy - previous_energy) / energy));
            if (rel < EPS) {
                reason = 2;
                break;
            }
            previous_energy = energy;
            const int nM = moving_pixels(S, prev);
            if ((float)nM / (float)S.N < PERCENT_MOVING) {
                reason = 3;
                break;
            }
            for (int c = 0; c < 3; ++c) prev[c] = S.U[c];
        }
        if (!cfg.early_exit || !cfg.faithful) continue;
        if ((double)energy < EPS) {
            if ((double)previous_energy_reweight < EPS) break;
            previous_energy_reweight = energy;
            continue;
        }
        const int nM = moving_pixels(S, prev_meta);
        if ((float)nM / (float)S.N < PERCENT_MOVING) break;
        for (int c = 0; c < 3; ++c) prev_meta[c] = S.U[c];
    }
    for (int c = 0; c < 3; ++c) std::copy(S.U[c].begin(), S.U[c].end(), out + c * S.N);
    if (st) {
        st->outer_iterations = total_k;
        st->meta_iterations = std::min(r + 1, cfg.nmeta_iter);
        st->stop_reason = reason;
        st->energy = (double)energy;
        st->gap = cfg.faithful ? 0.0 : tv_gap_last;
    }
}

// ------------------------------------------------------------------ IBR_gradient
// setup_target_visibility, sources/gradientIBR.cu:40-83 with setup_visibility_mask
// (sources/gradientIBR_kernels.cuh:4-55): a pixel is visible when some splatted tap has dx*dy != 0.
template <class T>
void gradient_visibility(const Problem<T> &P, uint8_t *vis) {
    std::fill(vis, vis + (size_t)P.W * P.H, 0);
    const int n = P.w * P.h;
    for (const auto &vw : P.views)
        for (int m = 0; m < n; ++m) {
            if (!in_splat(vw.tx[m], vw.ty[m], P.W, P.H)) continue;
            const Footprint<T> &fp = vw.fp[m];
            for (int j = 0; j < fp.ks; ++j)
                for (int i = 0; i < fp.ks; ++i) {
                    const int x = fp.x0 + j, y = fp.y0 + i;
                    if (0 <= x && x <= P.W - 1 && 0 <= y && y <= P.H - 1 &&
                        footprint_tap_nonzero(vw.tx[m], vw.ty[m], P.dsf, j, i, x, y))
                        vis[(size_t)y * P.W + x] = 1;
                }
        }
}

// hole_filling, sources/gradientIBR.cu:87-152, with compute_laplacian (sources/gradientIBR_kernels.cuh:
// 553-590): Jacobi diffusion of the holes, stop when the change of the last channel's sum(lap*U) < 1e-3.
template <class T>
int hole_fill(int W, int H, const uint8_t *vis, T *U, int max_iter) {
    const size_t N = (size_t)W * H;
    Vec<T> lap(N);
    T energy = 0, previous_energy = 0;
    int k;
    for (k = 0; k < max_iter; ++k) {
        previous_energy = energy;
        for (int c = 0; c < 3; ++c) {
            T *u = U + c * N;
#pragma omp parallel for
            for (int oy = 0; oy < H; ++oy)
                for (int ox = 0; ox < W; ++ox) {
                    const size_t o = (size_t)oy * W + ox;
                    if (vis[o]) {
                        lap[o] = 0;
                        continue;
                    }
                    T v = 0, wt = 0;
                    if (ox > 0) { v += u[o - 1]; wt += 1; }
                    if (oy > 0) { v += u[o - W]; wt += 1; }
                    if (ox < W - 1) { v += u[o + 1]; wt += 1; }
                    if (oy < H - 1) { v += u[o + W]; wt += 1; }
                    v /= wt;
                    v -= u[o];
                    lap[o] = v;
                }
            for (size_t o = 0; o < N; ++o) u[o] += lap[o];
            energy = 0;
            for (size_t o = 0; o < N; ++o) energy += lap[o] * u[o];
        }
        if (std::abs(previous_energy - energy) < (T)1e-3) return k + 1;
    }
    return k;
}

// init_u_gradient, sources/gradientIBR.cu:833-920: per view Sobel of the luminance (low res, no mask),
// splatted with A together with the view weights, normalised by the coverage; mask scaled by sigma^2.
template <class T>
void u_gradient(const Problem<T> &P, const lfrv_config &cfg, T *gx, T *gy, T *mask) {
    const size_t N = (size_t)P.W * P.H, n = (size_t)P.w * P.h;
    std::fill(gx, gx + N, T(0));
    std::fill(gy, gy + N, T(0));
    std::fill(mask, mask + N, T(0));
    Vec<T> norm(N, T(0)), vx(n), vy(n);
    for (const auto &vw : P.views) {
        sobel(P.w, P.h, vw.img, vw.img + n, vw.img + 2 * n, vx.data(), vy.data(), (const uint8_t *)nullptr);
        const T *in[3] = {vx.data(), vy.data(), vw.w.data()};
        T *out[3] = {gx, gy, mask};
        splat(P, vw, 3, in, out, norm.data(), (const T *)nullptr);
    }
    normalize(N, gx, norm.data());
    normalize(N, gy, norm.data());
    normalize(N, mask, norm.data());
    const T s2 = (T)cfg.sigma_sensor * (T)cfg.sigma_sensor;
    for (size_t o = 0; o < N; ++o) mask[o] *= s2;
}

// The Poisson operator of possion_conj_grad (updateAlpha, sources/solver.cu:201-310, lambda = 1):
// q = lambda d - Delta_N d with one-sided second differences at the borders.
template <class T>
inline T cg_op(const T *d, int W, int H, int ox, int oy, T lambda) {
    const size_t o = (size_t)oy * W + ox;
    T lx, ly;
    if (ox == 0) lx = d[o] - d[o + 1];
    else if (ox < W - 1) lx = 2 * d[o] - d[o - 1] - d[o + 1];
    else lx = d[o] - d[o - 1];
    if (oy == 0) ly = d[o] - d[o + W];
    else if (oy < H - 1) ly = 2 * d[o] - d[o - W] - d[o + W];
    else ly = d[o] - d[o - W];
    return lambda * d[o] + lx + ly;
}

// r0 = b - A x0 of initConjGrad (sources/solver.cu:361-505) for one channel.
template <class T>
inline T cg_r0(const T *u, const T *gX, const T *gY, int W, int H, int ox, int oy) {
    const size_t o = (size_t)oy * W + ox;
    T lx, ly;
    if (ox == 0) lx = u[o] - u[o + 1] + gX[o];
    else if (ox < W - 1) lx = 2 * u[o] - u[o - 1] - u[o + 1] + gX[o] - gX[o - 1];
    else lx = u[o] - u[o - 1] - gX[o - 1];
    if (oy == 0) ly = u[o] - u[o + W] + gY[o];
    else if (oy < H - 1) ly = 2 * u[o] - u[o - W] - u[o + W] + gY[o] - gY[o - W];
    else ly = u[o] - u[o - W] - gY[o - W];
    return -(lx + ly);
}

// Quadratic energy whose minimiser the CG computes: sum_c 1/2 lambda ||u_c - u0_c||^2 + 1/2 ||grad u_c - g||^2
// (forward differences where they exist), lambda = 1.
template <class T>
double cg_energy(int W, int H, const T *U, const T *U0, const T *gX, const T *gY) {
    const size_t N = (size_t)W * H;
    double e = 0;
    for (int c = 0; c < 3; ++c) {
        const T *u = U + c * N, *u0 = U0 + c * N;
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t o = (size_t)y * W + x;
                const double d = (double)u[o] - (double)u0[o];
                e += 0.5 * d * d;
                if (x < W - 1) {
                    const double a = (double)u[o + 1] - (double)u[o] - (double)gX[o];
                    e += 0.5 * a * a;
                }
                if (y < H - 1) {
                    const double a = (double)u[o + W] - (double)u[o] - (double)gY[o];
                    e += 0.5 * a * a;
                }
            }
    }
    return e;
}

// possion_conj_grad, sources/solver.cu:526-699.
//   faithful: the reference's loop (5 iterations; beta == 1 because deltaNew is never refreshed; the
//             alpha accumulator dAlpha is never cleared and also receives r.r from updateSolution; the
//             last image row's r.r counted twice at init). The reference's uninitialised read in that
//             double count and its read of alpha while other blocks add into it are resolved as: the
//             second count uses the row's correct residual, and alpha is read before any addition.
//   corrected: conjugate gradient per channel with double dot products, stopping when the certified
//             relative gap ||r||^2/(2 lambda) / (E(u) - ||r||^2/(2 lambda)) <= gap_tol or at max_iter.
// trace (optional, trace_cap entries): the energy after each iteration -- the FP64 quadratic energy of the
// iterate (faithful) or the energy lowered by each step's decrease (corrected), as the device solvers record it.
template <class T>
int cg_solve(int W, int H, bool faithful, int max_iter, double gap_tol, const T *gX, const T *gY, T *U,
             double *gap_out, double *trace = nullptr, int trace_cap = 0) {
    const size_t N = (size_t)W * H;
    const T lambda = 1;
    Vec<T> U0(U, U + 3 * N);
    Vec<T> r(3 * N), d(3 * N), q(3 * N);
    double delta[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) {
        const T *u = U + c * N;
        T *rc = r.data() + c * N;
        double dl = 0;
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t o = (size_t)y * W + x;
                rc[o] = cg_r0(u, gX, gY, W, H, x, y);
                dl += (double)rc[o] * (double)rc[o];
                if (faithful && y == H - 1) dl += (double)rc[o] * (double)rc[o];
            }
        delta[c] = dl;
    }
    d = r;
    int it = 0;
    if (faithful) {
        const int nIter = 5;
        double dAlpha[3] = {0, 0, 0};
        for (it = 0; it < nIter; ++it) {
            for (int c = 0; c < 3; ++c) {
                T *dc = d.data() + c * N, *qc = q.data() + c * N;
                double dq = 0;
                for (int y = 0; y < H; ++y)
                    for (int x = 0; x < W; ++x) {
                        const size_t o = (size_t)y * W + x;
                        qc[o] = cg_op(dc, W, H, x, y, lambda);
                        dq += (double)dc[o] * (double)qc[o];
                    }
                dAlpha[c] += dq;
                const T alpha = (T)((float)delta[c] / (float)dAlpha[c]);
                T *u = U + c * N, *rc = r.data() + c * N;
                double rr = 0;
                for (size_t o = 0; o < N; ++o) {
                    u[o] += alpha * dc[o];
                    rc[o] -= alpha * qc[o];
                    rr += (double)rc[o] * (double)rc[o];
                }
                dAlpha[c] = (double)alpha + rr;  // updateSolution adds r.r into the alpha slot
                for (size_t o = 0; o < N; ++o) dc[o] = rc[o] + (T)1 * dc[o];  // beta = deltaNew/deltaOld = 1
            }
            if (trace && it < trace_cap) trace[it] = cg_energy(W, H, U, U0.data(), gX, gY);
        }
        if (gap_out) *gap_out = 0;
        return it;
    }
    // E(x_{k+1}) = E(x_k) - alpha_k delta_k / 2 along CG steps (d_k . r_k = r_k . r_k); the certificate
    // E(x) - E* = r^T A^-1 r / 2 <= ||r||^2 / (2 lambda) since A >= lambda I.
    double E = cg_energy(W, H, U, U0.data(), gX, gY);
    double gap = 1e300;
    for (it = 0;; ++it) {
        const double bound = (delta[0] + delta[1] + delta[2]) / (2.0 * (double)lambda);
        gap = (E - bound) > 0 ? bound / (E - bound) : 1e300;
        if (it >= max_iter || (gap_tol > 0 && gap <= gap_tol)) break;
        for (int c = 0; c < 3; ++c) {
            T *dc = d.data() + c * N, *qc = q.data() + c * N;
            double dq = 0;
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x) {
                    const size_t o = (size_t)y * W + x;
                    qc[o] = cg_op(dc, W, H, x, y, lambda);
                    dq += (double)dc[o] * (double)qc[o];
                }
            if (!(dq > 0)) continue;
            const double alpha = delta[c] / dq;
            T *u = U + c * N, *rc = r.data() + c * N;
            double rr = 0;
            for (size_t o = 0; o < N; ++o) {
                u[o] += (T)alpha * dc[o];
                rc[o] -= (T)alpha * qc[o];
                rr += (double)rc[o] * (double)rc[o];
            }
            E -= 0.5 * alpha * delta[c];
            const double beta = rr / delta[c];
            delta[c] = rr;
            for (size_t o = 0; o < N; ++o) dc[o] = rc[o] + (T)beta * dc[o];
        }
        if (trace && it < trace_cap) trace[it] = E;
    }
    if (gap_out) *gap_out = gap;
    return it;
}

// poisson_jacobi, sources/gradientIBR.cu:923-1013 (the Jacobi alternative to the CG, left commented out at
// sources/gradientIBR.cpp:131): per channel z = (lambda m u0 - div g) / (4 + lambda m) with lambda = 1, m the target
// mask and div the central-difference divergence of compute_divergence (sources/gradientIBR_kernels.cuh:553-575,
// zero on the border rows / columns), jacobi_z (:577-598); then `iters` sweeps (200 upstream) of jacobi_B (:600-643):
// x <- (x_left + x_up + x_right + x_down) / (4 + lambda m) + z, the border pixel standing in for a missing neighbour.
template <class T>
void poisson_jacobi(int W, int H, const T *gX, const T *gY, const T *mask, T *U, int iters) {
    const size_t N = (size_t)W * H;
    const T lambda = (T)1.0;
    Vec<T> z(3 * N), tmp(N);
    for (int c = 0; c < 3; ++c)
        for (int oy = 0; oy < H; ++oy)
            for (int ox = 0; ox < W; ++ox) {
                const size_t o = (size_t)oy * W + ox;
                T dv = 0;
                if (ox != 0 && ox != W - 1) dv += (gX[o + 1] - gX[o - 1]) / 2;
                if (oy != 0 && oy != H - 1) dv += (gY[o + W] - gY[o - W]) / 2;
                const T data_w = lambda * mask[o];
                z[c * N + o] = (data_w * U[c * N + o] - dv) / (4 + data_w);
            }
    for (int k = 0; k < iters; ++k)
        for (int c = 0; c < 3; ++c) {
            T *u = U + c * N;
            std::copy(u, u + N, tmp.begin());
#pragma omp parallel for
            for (int oy = 0; oy < H; ++oy)
                for (int ox = 0; ox < W; ++ox) {
                    const size_t o = (size_t)oy * W + ox;
                    T x = 0;
                    x += ox == 0 ? tmp[o] : tmp[o - 1];
                    x += oy == 0 ? tmp[o] : tmp[o - W];
                    x += ox == W - 1 ? tmp[o] : tmp[o + 1];
                    x += oy == H - 1 ? tmp[o] : tmp[o + W];
                    x /= (4 + lambda * mask[o]);
                    x += z[c * N + o];
                    u[o] = x;
                }
        }
}

// IBR_gradient, sources/gradientIBR.cpp:12-150.
template <class T>
void ibr_gradient(const lfrv_config &cfg, const T *views, const T *tau, int tau_ch, const T *dpart, const T *init,
                  T *out, lfrv_stats *st) {
    Problem<T> P;
    build_problem(P, cfg, views, tau, tau_ch, dpart);
    const size_t N = (size_t)P.W * P.H, n = (size_t)P.w * P.h;
    std::vector<uint8_t> vis(N);
    gradient_visibility(P, vis.data());
    // compute_weights (sources/gradientIBR.cu:558-648) with U = 0: unmasked Sobel of 0 is 0.
    Vec<T> U(3 * N, T(0)), zx(N, T(0)), zy(N, T(0));
    for (auto &vw : P.views) view_weights(P, vw, zx.data(), zy.data(), (T)cfg.sigma_sensor, (T)cfg.ugrad_threshold);
    int hf = 0;
    if (init) {
        std::copy(init, init + 3 * N, U.begin());
    } else {
        // compute_initial_image (sources/gradientIBR.cu:724-808)
        Vec<T> norm(N, T(0));
        for (auto &vw : P.views) {
            const T *in[3] = {vw.img, vw.img + n, vw.img + 2 * n};
            T *o3[3] = {U.data(), U.data() + N, U.data() + 2 * N};
            splat(P, vw, 3, in, o3, norm.data(), vw.w.data());
        }
        for (int c = 0; c < 3; ++c) normalize(N, U.data() + c * N, norm.data());
        hf = hole_fill(P.W, P.H, vis.data(), U.data(), cfg.hole_fill_iter);
    }
    Vec<T> gx(N), gy(N), mask(N);
    u_gradient(P, cfg, gx.data(), gy.data(), mask.data());
    double gap = 0;
    const bool traced = st && st->energy_trace && st->trace_capacity > 0;
    const int it = cg_solve(P.W, P.H, cfg.faithful != 0, cfg.cg_max_iter, cfg.cg_gap_tol, gx.data(), gy.data(),
                            U.data(), &gap, traced ? st->energy_trace : nullptr, traced ? st->trace_capacity : 0);
    std::copy(U.begin(), U.end(), out);
    if (st) {
        st->trace_length = traced ? std::min(it, st->trace_capacity) : 0;
        st->outer_iterations = it;
        st->hole_fill_iterations = hf;
        st->gap = gap;
        st->stop_reason = (!cfg.faithful && cfg.cg_gap_tol > 0 && gap <= cfg.cg_gap_tol) ? 4 : 0;
    }
}

// ------------------------------------------------------------------ warp stage (GLSL restated)
struct Cam {
    double K[9], R[9], t[3], Kinv[9];
    int W, H;
};

inline void inv3(const double *m, double *o) {
    const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double det = a * A + b * B + c * C;
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

inline Cam to_cam(const lfrv_camera &c) {
    Cam k;
    for (int i = 0; i < 9; ++i) {
        k.K[i] = c.K[i];
        k.R[i] = c.R[i];
    }
    for (int i = 0; i < 3; ++i) k.t[i] = c.t[i];
    inv3(k.K, k.Kinv);
    k.W = c.width;
    k.H = c.height;
    return k;
}

inline void mv(const double *M, const double *x, double *y) {
    for (int r = 0; r < 3; ++r) y[r] = M[3 * r] * x[0] + M[3 * r + 1] * x[1] + M[3 * r + 2] * x[2];
}
inline void mtv(const double *M, const double *x, double *y) {  // M^T x
    for (int r = 0; r < 3; ++r) y[r] = M[r] * x[0] + M[3 + r] * x[1] + M[6 + r] * x[2];
}

// X = R^T (K^-1 (z * (x, y, 1)) - t): the unprojection of tauWarp.frag:31 and depthSplatting.geom:31.
inline void unproject(const Cam &c, double x, double y, double z, double *X) {
    const double p[3] = {z * x, z * y, z};
    double q[3];
    mv(c.Kinv, p, q);
    for (int i = 0; i < 3; ++i) q[i] -= c.t[i];
    mtv(c.R, q, X);
}
// x_h = K (R X + t) (tauWarp.frag:32)
inline void project(const Cam &c, const double *X, double *xh) {
    double q[3];
    mv(c.R, X, q);
    for (int i = 0; i < 3; ++i) q[i] += c.t[i];
    mv(c.K, q, xh);
}

// Target depth map (Scene::computeTargetDepthMap sources/openGL/scene.cpp:1506-1544 driving
// depthSplatting.{vert,geom,frag}): every input pixel with z < INVALID_DEPTH/2 becomes a quad with
// corners (x +- 1/2, y +- 1/2) at depths z +- dz/dx/2 +- dz/dy/2 (geom :36-58), drawn as the strip
// BL, TL, BR, TR. A target pixel centre covered by a triangle (top-left fill rule) keeps the quad with
// the smallest depth interpolated linearly in screen space in 1/z (the perspective depth the GL depth
// test compares) and stores the quad CENTRE's target depth (depthSplatting.frag:13-15). Uncovered
// pixels hold 0 (the colour clear value, scene.cpp:1515).
inline double edge(double ax, double ay, double bx, double by, double px, double py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
inline bool top_left(double ax, double ay, double bx, double by, bool ccw) {
    // For counter-clockwise (positive area in y-down pixel space) triangles an edge is "top" when it is
    // horizontal with the interior below, "left" when it goes down.
    const double ex = bx - ax, ey = by - ay;
    if (!ccw) return (ey == 0 && ex < 0) || ey > 0;
    return (ey == 0 && ex > 0) || ey < 0;
}

inline void raster_tri(const double *v0, const double *v1, const double *v2, double zc, int W, int H,
                       std::vector<double> &best, std::vector<double> &val) {
    double area = edge(v0[0], v0[1], v1[0], v1[1], v2[0], v2[1]);
    if (area == 0) return;
    const bool ccw = area > 0;
    const int xmin = std::max(0, (int)std::floor(std::min({v0[0], v1[0], v2[0]}) - 0.5));
    const int xmax = std::min(W - 1, (int)std::ceil(std::max({v0[0], v1[0], v2[0]}) - 0.5));
    const int ymin = std::max(0, (int)std::floor(std::min({v0[1], v1[1], v2[1]}) - 0.5));
    const int ymax = std::min(H - 1, (int)std::ceil(std::max({v0[1], v1[1], v2[1]}) - 0.5));
    if (xmax < xmin || ymax < ymin) return;
    if (xmax - xmin > 64 || ymax - ymin > 64) return;  // degenerate (grazing) quads are skipped
    const bool tl0 = top_left(v1[0], v1[1], v2[0], v2[1], ccw);
    const bool tl1 = top_left(v2[0], v2[1], v0[0], v0[1], ccw);
    const bool tl2 = top_left(v0[0], v0[1], v1[0], v1[1], ccw);
    for (int y = ymin; y <= ymax; ++y)
        for (int x = xmin; x <= xmax; ++x) {
            const double px = x + 0.5, py = y + 0.5;
            double w0 = edge(v1[0], v1[1], v2[0], v2[1], px, py);
            double w1 = edge(v2[0], v2[1], v0[0], v0[1], px, py);
            double w2 = edge(v0[0], v0[1], v1[0], v1[1], px, py);
            if (!ccw) {
                w0 = -w0;
                w1 = -w1;
                w2 = -w2;
            }
            if (w0 < 0 || w1 < 0 || w2 < 0) continue;
            if ((w0 == 0 && !tl0) || (w1 == 0 && !tl1) || (w2 == 0 && !tl2)) continue;
            const double s = w0 + w1 + w2;
            const double iz = (w0 * v0[2] + w1 * v1[2] + w2 * v2[2]) / s;  // interpolated 1/z
            const size_t o = (size_t)y * W + x;
            if (iz > best[o] || (iz == best[o] && zc < val[o])) {
                best[o] = iz;
                val[o] = zc;
            }
        }
}

inline void zbuffer(int V, int w, int h, const float *depth, const Cam *cams, const Cam &u, float *zbuf) {
    const int W = u.W, H = u.H;
    std::vector<double> best((size_t)W * H, 0.0), val((size_t)W * H, 0.0);
    const size_t n = (size_t)w * h;
    for (int v = 0; v < V; ++v) {
        const float *dz = depth + (size_t)v * 3 * n;
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const size_t m = (size_t)y * w + x;
                const double z = dz[m], zx = dz[n + m], zy = dz[2 * n + m];
                if (z >= kInvalidDepth / 2) continue;
                const double cx = x + 0.5, cy = y + 0.5;
                double X[3], xh[3];
                unproject(cams[v], cx, cy, z, X);
                project(u, X, xh);
                const double zc = xh[2];
                const double off[4][2] = {{-0.5, -0.5}, {-0.5, 0.5}, {0.5, -0.5}, {0.5, 0.5}};  // BL TL BR TR
                double vert[4][3];
                bool ok = true;
                for (int k = 0; k < 4; ++k) {
                    const double dx = off[k][0], dy = off[k][1];
                    const double zk = z + dx * zx + dy * zy;
                    unproject(cams[v], cx + dx, cy + dy, zk, X);
                    project(u, X, xh);
                    if (!(xh[2] > 1e-2)) ok = false;  // behind the near plane (zNear = 1e-2, pinholeCamera.cpp:133)
                    vert[k][0] = xh[0] / xh[2];
                    vert[k][1] = xh[1] / xh[2];
                    vert[k][2] = 1.0 / xh[2];
                }
                if (!ok) continue;
                raster_tri(vert[0], vert[1], vert[2], zc, W, H, best, val);
                raster_tri(vert[1], vert[2], vert[3], zc, W, H, best, val);
            }
    }
    for (size_t o = 0; o < (size_t)W * H; ++o) zbuf[o] = (float)val[o];
}

// GL_LINEAR lookup of a sampler2DRect with CLAMP_TO_EDGE (sources/openGL/texture.cpp:153-156): texel
// centres at i + 1/2.
inline double bilinear(const float *img, int W, int H, double u, double v) {
    const double fx = u - 0.5, fy = v - 0.5;
    const int x0 = (int)std::floor(fx), y0 = (int)std::floor(fy);
    const double ax = fx - x0, ay = fy - y0;
    auto at = [&](int x, int y) {
        x = std::min(std::max(x, 0), W - 1);
        y = std::min(std::max(y, 0), H - 1);
        return (double)img[(size_t)y * W + x];
    };
    return (1 - ay) * ((1 - ax) * at(x0, y0) + ax * at(x0 + 1, y0)) + ay * ((1 - ax) * at(x0, y0 + 1) + ax * at(x0 + 1, y0 + 1));
}

// tauWarp.frag:25-74 and tauPartial.frag:23-48 for one input pixel.
inline void tau_pixel(const Cam &k, const Cam &u, const float *zbuf, double x, double y, double z, double zx,
                      double zy, float *tau3, float *dpart3) {
    double X[3], xuh[3];
    unproject(k, x, y, z, X);
    project(u, X, xuh);
    double xu = 0, yu = 0;
    if (xuh[2] != 0) {
        xu = xuh[0] / xuh[2];
        yu = xuh[1] / xuh[2];
    }
    // M = K_u R_u R_k^T K_k^-1 (3x3)
    double M[9], RtKi[9], RuRt[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int q = 0; q < 3; ++q) s += k.R[3 * q + r] * k.Kinv[3 * q + c];  // R_k^T K_k^-1
            RtKi[3 * r + c] = s;
        }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int q = 0; q < 3; ++q) s += u.R[3 * r + q] * RtKi[3 * q + c];
            RuRt[3 * r + c] = s;
        }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int q = 0; q < 3; ++q) s += u.K[3 * r + q] * RuRt[3 * q + c];
            M[3 * r + c] = s;
        }
    // Je = [[1, 0, -xu], [0, 1, -yu]] / xuh.z
    auto Je_apply = [&](const double *v3, double *o2) {
        o2[0] = (v3[0] - xu * v3[2]) / xuh[2];
        o2[1] = (v3[1] - yu * v3[2]) / xuh[2];
    };
    // deformation: columns (x dzdx + z, y dzdx, dzdx) and (x dzdy, y dzdy + z, dzdy)
    const double c0[3] = {x * zx + z, y * zx, zx}, c1[3] = {x * zy, y * zy + z, zy};
    double m0[3], m1[3], d0[2], d1[2];
    mv(M, c0, m0);
    mv(M, c1, m1);
    Je_apply(m0, d0);
    Je_apply(m1, d1);
    double deform = 1.0 / std::fabs(d0[0] * d1[1] - d0[1] * d1[0]);
    if (deform >= 30.0) deform = 30.0;
    const double u_depth = bilinear(zbuf, u.W, u.H, xu, yu);
    if (xu <= 0 || u.W <= xu || yu <= 0 || u.H <= yu || z >= kInvalidDepth / 2) {
        tau3[0] = -2.0f;
        tau3[1] = -2.0f;
        tau3[2] = 0.0f;
    } else if (xuh[2] > u_depth + 0.10) {
        tau3[0] = -1.0f;
        tau3[1] = -1.0f;
        tau3[2] = 0.0f;
    } else {
        tau3[0] = (float)xu;
        tau3[1] = (float)yu;
        tau3[2] = (float)deform;
    }
    const double xk[3] = {x, y, 1.0};
    double mk[3], res[2];
    mv(M, xk, mk);
    Je_apply(mk, res);
    dpart3[0] = 10.0f;
    dpart3[1] = (float)res[0];
    dpart3[2] = (float)res[1];
}

}  // namespace orc

// ====================================================================== C exports
namespace {

template <class T>
std::vector<T> conv(const float *p, size_t n) {
    return p ? std::vector<T>(p, p + n) : std::vector<T>();
}
template <class T>
void back(const std::vector<T> &v, float *p) {
    if (p)
        for (size_t i = 0; i < v.size(); ++i) p[i] = (float)v[i];
}

template <class T>
int ibr_color_t(const lfrv_config *cfg, const float *views, const float *tau, int tau_ch, const float *dpart,
                const float *init, float *out, lfrv_stats *st) {
    const size_t n = (size_t)cfg->w * cfg->h, N = n * cfg->dsf * cfg->dsf, V = cfg->nviews;
    auto v = conv<T>(views, V * 3 * n), t = conv<T>(tau, V * tau_ch * n), d = conv<T>(dpart, V * 3 * n);
    auto i0 = conv<T>(init, 3 * N);
    std::vector<T> o(3 * N);
    orc::ibr_color<T>(*cfg, v.data(), t.data(), tau_ch, dpart ? d.data() : nullptr, init ? i0.data() : nullptr,
                      o.data(), st);
    back(o, out);
    return 0;
}

template <class T>
int ibr_gradient_t(const lfrv_config *cfg, const float *views, const float *tau, int tau_ch, const float *dpart,
                   const float *init, float *out, lfrv_stats *st) {
    const size_t n = (size_t)cfg->w * cfg->h, N = n * cfg->dsf * cfg->dsf, V = cfg->nviews;
    auto v = conv<T>(views, V * 3 * n), t = conv<T>(tau, V * tau_ch * n), d = conv<T>(dpart, V * 3 * n);
    auto i0 = conv<T>(init, 3 * N);
    std::vector<T> o(3 * N);
    orc::ibr_gradient<T>(*cfg, v.data(), t.data(), tau_ch, dpart ? d.data() : nullptr, init ? i0.data() : nullptr,
                         o.data(), st);
    back(o, out);
    return 0;
}

template <class T>
void make_color_state(orc::ColorState<T> &S, const lfrv_config *cfg, std::vector<T> &v, std::vector<T> &t,
                      std::vector<T> &d, const float *views, const float *tau, int tau_ch, const float *dpart) {
    const size_t n = (size_t)cfg->w * cfg->h, V = cfg->nviews;
    v = conv<T>(views, V * 3 * n);
    t = conv<T>(tau, V * tau_ch * n);
    d = conv<T>(dpart, V * 3 * n);
    S.init(*cfg, v.data(), t.data(), tau_ch, dpart ? d.data() : nullptr);
}

}  // namespace

#define ORC_DISPATCH(prec, fn, ...) ((prec) == 0 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

extern "C" {

int orc_ibr_color(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                  const float *dpart, const float *init, float *out, lfrv_stats *st) {
    return ORC_DISPATCH(prec, ibr_color_t, cfg, views, tau, tau_ch, dpart, init, out, st);
}

int orc_ibr_gradient(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                     const float *dpart, const float *init, float *out, lfrv_stats *st) {
    return ORC_DISPATCH(prec, ibr_gradient_t, cfg, views, tau, tau_ch, dpart, init, out, st);
}

// Visibility (IBR_color): coverage and mask.
int orc_stage_visibility(int prec, const lfrv_config *cfg, const float *tau, int tau_ch, float *coverage,
                         uint8_t *vis) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::ColorState<T> S;
        std::vector<T> v, t, d;
        const size_t n = (size_t)cfg->w * cfg->h;
        std::vector<float> dummy_views((size_t)cfg->nviews * 3 * n, 0.0f);
        make_color_state(S, cfg, v, t, d, dummy_views.data(), tau, tau_ch, nullptr);
        orc::color_visibility(S);
        back(S.cov, coverage);
        if (vis) std::copy(S.vis.begin(), S.vis.end(), vis);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

// Weights with explicit gradient buffers (see lfrv_stage_weights).
int orc_stage_weights(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                      const float *dpart, const float *U, const uint8_t *vis, float *gx, float *gy,
                      float *weights) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::ColorState<T> S;
        std::vector<T> v, t, d;
        make_color_state(S, cfg, v, t, d, views, tau, tau_ch, dpart);
        for (int c = 0; c < 3; ++c)
            for (size_t o = 0; o < S.N; ++o) S.U[c][o] = (T)U[c * S.N + o];
        for (size_t o = 0; o < S.N; ++o) {
            S.vis[o] = vis[o];
            S.X1[0][o] = (T)gx[o];
            S.X2[0][o] = (T)gy[o];
        }
        orc::color_compute_weights(S);
        back(S.X1[0], gx);
        back(S.X2[0], gy);
        const size_t n = (size_t)cfg->w * cfg->h;
        for (int vv = 0; vv < cfg->nviews; ++vv)
            for (size_t m = 0; m < n; ++m) weights[vv * n + m] = (float)S.P.views[vv].w[m];
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

// Data term G (before clamp) and F.
int orc_stage_dataterm(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                       const float *weights, const float *U, float *G, float *F) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::ColorState<T> S;
        std::vector<T> v, t, d;
        make_color_state(S, cfg, v, t, d, views, tau, tau_ch, nullptr);
        const size_t n = (size_t)cfg->w * cfg->h;
        for (int vv = 0; vv < cfg->nviews; ++vv)
            for (size_t m = 0; m < n; ++m) S.P.views[vv].w[m] = (T)weights[vv * n + m];
        for (int c = 0; c < 3; ++c)
            for (size_t o = 0; o < S.N; ++o) {
                S.U[c][o] = (T)U[c * S.N + o];
                S.G[c][o] = 0;
            }
        std::vector<T> gi(3 * S.N);
        T *gp[3] = {gi.data(), gi.data() + S.N, gi.data() + 2 * S.N};
        if (cfg->dt_alpha > 0) orc::color_dataterm(S, gp);
        if (cfg->dt_beta > 0) orc::color_dataterm_gradients(S);
        const orc::RofConsts<T> k = orc::rof_consts<T>(*cfg);
        for (int c = 0; c < 3; ++c)
            for (size_t o = 0; o < S.N; ++o) {
                G[c * S.N + o] = (float)S.G[c][o];
                T gv = std::min((T)1.0f, std::max((T)-1.0f, S.G[c][o]));
                gv *= k.fscale;
                gv += S.U[c][o];
                F[c * S.N + o] = (float)std::min((T)1.0f, std::max((T)0.0f, gv));
            }
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_rof(int prec, int W, int H, int niter, float tau, float sigma, float lam, const float *F,
                  const float *g, float *U, float *P) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        const size_t N = (size_t)W * H;
        std::vector<T> f = conv<T>(F, 3 * N), gg = conv<T>(g, N), u = conv<T>(U, 3 * N), p = conv<T>(P, 6 * N);
        const T *Fp[3] = {f.data(), f.data() + N, f.data() + 2 * N};
        T *Up[3] = {u.data(), u.data() + N, u.data() + 2 * N};
        T *PX[3] = {p.data(), p.data() + 2 * N, p.data() + 4 * N};
        T *PY[3] = {p.data() + N, p.data() + 3 * N, p.data() + 5 * N};
        orc::rof_iterations<T>(W, H, niter, (T)tau, (T)sigma, (T)lam, Fp, gg.data(), Up, PX, PY);
        back(u, U);
        back(p, P);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_energy(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                     const float *weights, const float *U, const uint8_t *vis, double *energy, double *e_tv,
                     double *e_data) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::ColorState<T> S;
        std::vector<T> v, t, d;
        make_color_state(S, cfg, v, t, d, views, tau, tau_ch, nullptr);
        const size_t n = (size_t)cfg->w * cfg->h;
        for (int vv = 0; vv < cfg->nviews; ++vv)
            for (size_t m = 0; m < n; ++m) S.P.views[vv].w[m] = (T)weights[vv * n + m];
        for (int c = 0; c < 3; ++c)
            for (size_t o = 0; o < S.N; ++o) S.U[c][o] = (T)U[c * S.N + o];
        for (size_t o = 0; o < S.N; ++o) S.vis[o] = vis[o];
        T et, ed;
        const T e = orc::color_energy(S, &et, &ed);
        if (energy) *energy = (double)e;
        if (e_tv) *e_tv = (double)et;
        if (e_data) *e_data = (double)ed;
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_regularizer(int prec, const lfrv_config *cfg, const float *tau, int tau_ch, const float *weights,
                          const float *norm_in, float *norm_out, float *g) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::ColorState<T> S;
        std::vector<T> v, t, d;
        const size_t n = (size_t)cfg->w * cfg->h;
        std::vector<float> dummy_views((size_t)cfg->nviews * 3 * n, 0.0f);
        make_color_state(S, cfg, v, t, d, dummy_views.data(), tau, tau_ch, nullptr);
        for (int vv = 0; vv < cfg->nviews; ++vv)
            for (size_t m = 0; m < n; ++m) S.P.views[vv].w[m] = (T)weights[vv * n + m];
        for (size_t o = 0; o < S.N; ++o) S.norm_mask[o] = norm_in ? (T)norm_in[o] : T(0);
        orc::color_regularizer(S);
        back(S.norm_mask, norm_out);
        back(S.g, g);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_initial_image(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                            const float *weights, float *U, float *norm) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::ColorState<T> S;
        std::vector<T> v, t, d;
        make_color_state(S, cfg, v, t, d, views, tau, tau_ch, nullptr);
        const size_t n = (size_t)cfg->w * cfg->h;
        for (int vv = 0; vv < cfg->nviews; ++vv)
            for (size_t m = 0; m < n; ++m) S.P.views[vv].w[m] = (T)weights[vv * n + m];
        orc::color_initial_image(S, false);
        for (int c = 0; c < 3; ++c)
            for (size_t o = 0; o < S.N; ++o) U[c * S.N + o] = (float)S.U[c][o];
        back(S.norm_mask, norm);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_push_pull(int prec, int W, int H, int faithful, const uint8_t *vis, float *U) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        std::vector<T> u = conv<T>(U, 3 * (size_t)W * H);
        orc::push_pull<T>(W, H, vis, u.data(), faithful != 0);
        back(u, U);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_gradient_visibility(int prec, const lfrv_config *cfg, const float *tau, int tau_ch, uint8_t *vis) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::Problem<T> P;
        const size_t n = (size_t)cfg->w * cfg->h;
        std::vector<T> v((size_t)cfg->nviews * 3 * n, T(0)), t = conv<T>(tau, (size_t)cfg->nviews * tau_ch * n);
        orc::build_problem(P, *cfg, v.data(), t.data(), tau_ch, (const T *)nullptr);
        orc::gradient_visibility(P, vis);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_hole_fill(int prec, int W, int H, int max_iter, const uint8_t *vis, float *U, int *iterations) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        std::vector<T> u = conv<T>(U, 3 * (size_t)W * H);
        const int it = orc::hole_fill<T>(W, H, vis, u.data(), max_iter);
        if (iterations) *iterations = it;
        back(u, U);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_u_gradient(int prec, const lfrv_config *cfg, const float *views, const float *tau, int tau_ch,
                         const float *weights, float *gx, float *gy, float *mask) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        orc::Problem<T> P;
        const size_t n = (size_t)cfg->w * cfg->h, N = n * cfg->dsf * cfg->dsf;
        std::vector<T> v = conv<T>(views, (size_t)cfg->nviews * 3 * n), t = conv<T>(tau, (size_t)cfg->nviews * tau_ch * n);
        orc::build_problem(P, *cfg, v.data(), t.data(), tau_ch, (const T *)nullptr);
        for (int vv = 0; vv < cfg->nviews; ++vv)
            for (size_t m = 0; m < n; ++m) P.views[vv].w[m] = (T)weights[vv * n + m];
        std::vector<T> a(N), b(N), c(N);
        orc::u_gradient(P, *cfg, a.data(), b.data(), c.data());
        back(a, gx);
        back(b, gy);
        back(c, mask);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_cg(int prec, int W, int H, int faithful, int max_iter, double gap_tol, const float *gx,
                 const float *gy, float *U, int *iterations, double *gap) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        const size_t N = (size_t)W * H;
        std::vector<T> a = conv<T>(gx, N), b = conv<T>(gy, N), u = conv<T>(U, 3 * N);
        const int it = orc::cg_solve<T>(W, H, faithful != 0, max_iter, gap_tol, a.data(), b.data(), u.data(), gap);
        if (iterations) *iterations = it;
        back(u, U);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_stage_poisson_jacobi(int prec, int W, int H, int iters, const float *gx, const float *gy, const float *mask,
                             float *U) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        const size_t N = (size_t)W * H;
        std::vector<T> a = conv<T>(gx, N), b = conv<T>(gy, N), m = conv<T>(mask, N), u = conv<T>(U, 3 * N);
        orc::poisson_jacobi<T>(W, H, a.data(), b.data(), m.data(), u.data(), iters);
        back(u, U);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

double orc_cg_energy(int W, int H, const float *U, const float *U0, const float *gx, const float *gy) {
    return orc::cg_energy<float>(W, H, U, U0, gx, gy);
}

// Warp stage: target z-buffer, tau (3 ch) and dpart (3 ch) per view. FP64 only.
int orc_warp(int V, int w, int h, const float *depth, const lfrv_camera *cams, const lfrv_camera *target, float *tau,
             float *dpart, float *zbuf) {
    std::vector<orc::Cam> ks(V);
    for (int v = 0; v < V; ++v) ks[v] = orc::to_cam(cams[v]);
    const orc::Cam u = orc::to_cam(*target);
    std::vector<float> zb((size_t)u.W * u.H);
    orc::zbuffer(V, w, h, depth, ks.data(), u, zb.data());
    if (zbuf) std::copy(zb.begin(), zb.end(), zbuf);
    const size_t n = (size_t)w * h;
    for (int v = 0; v < V; ++v) {
        const float *dz = depth + (size_t)v * 3 * n;
        float *tv = tau ? tau + (size_t)v * 3 * n : nullptr;
        float *dv = dpart ? dpart + (size_t)v * 3 * n : nullptr;
#pragma omp parallel for
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const size_t m = (size_t)y * w + x;
                float t3[3], d3[3];
                orc::tau_pixel(ks[v], u, zb.data(), x + 0.5, y + 0.5, dz[m], dz[n + m], dz[2 * n + m], t3, d3);
                if (tv)
                    for (int c = 0; c < 3; ++c) tv[c * n + m] = t3[c];
                if (dv)
                    for (int c = 0; c < 3; ++c) dv[c * n + m] = d3[c];
            }
    }
    return 0;
}

// import_warps_from_depth, sources/import.cpp:243-450: warps from orthographic depth maps and cameras without
// the GL pipeline, in float like the reference's glm arithmetic. Pass 1 projects every source pixel into the
// target (tau = x_h / z_h) and keeps, over the dsf x dsf pixels from int(tau) - dsf/2, the smallest target depth
// z_h. Pass 2 averages that depth map over the pixel's footprint (overlaps dx dy, INVALID_DEPTH texels skipped),
// back-projects the nearest target pixel with it and marks the warp (-2w, -2h) when the result lands more than
// 10 pixels from the source pixel; no coverage gives (-w, -h). Faithful mode back-projects with the source
// camera's R and C (the reference passes v_i_cam's, import.cpp:412-415); otherwise with the target's.
// tau: V x 3 x n (tau_x, tau_y, tau_y as the reference writes it).
namespace orc {
struct GlmCam {
    float fx, fy, cx, cy;  // K entries the reference uses for K^-1
    float R[9], C[3], P[12];  // row-major R, centre, P = K [R | t] in float
};
inline GlmCam glm_cam(const lfrv_camera &c) {
    GlmCam g;
    g.fx = c.K[0];
    g.fy = c.K[4];
    g.cx = c.K[2];
    g.cy = c.K[5];
    for (int i = 0; i < 9; ++i) g.R[i] = c.R[i];
    for (int r = 0; r < 3; ++r) g.C[r] = -(c.R[0 * 3 + r] * c.t[0] + c.R[1 * 3 + r] * c.t[1] + c.R[2 * 3 + r] * c.t[2]);
    for (int r = 0; r < 3; ++r) {
        for (int col = 0; col < 3; ++col)
            g.P[r * 4 + col] = c.K[r * 3 + 0] * c.R[0 * 3 + col] + c.K[r * 3 + 1] * c.R[1 * 3 + col] +
                               c.K[r * 3 + 2] * c.R[2 * 3 + col];
        g.P[r * 4 + 3] = c.K[r * 3 + 0] * c.t[0] + c.K[r * 3 + 1] * c.t[1] + c.K[r * 3 + 2] * c.t[2];
    }
    return g;
}
// X = d K^-1 (px, py, 1) with K^-1 = [[1/fx, 0, -cx/fx], [0, 1/fy, -cy/fy], [0, 0, 1]]; world = R^T X + C of `rc`;
// then projected with `pc`: out = P (world, 1).
inline void wfd_transfer(const GlmCam &kc, const GlmCam &rc, const GlmCam &pc, float d, float px, float py,
                         float out[3]) {
    const float i00 = (float)(1.0 / kc.fx), i11 = (float)(1.0 / kc.fy), i20 = -kc.cx / kc.fx, i21 = -kc.cy / kc.fy;
    const float X[3] = {d * i00 * px + d * i20, d * i11 * py + d * i21, d};
    float Xw[3];
    for (int r = 0; r < 3; ++r) Xw[r] = rc.R[0 * 3 + r] * X[0] + rc.R[1 * 3 + r] * X[1] + rc.R[2 * 3 + r] * X[2] + rc.C[r];
    for (int r = 0; r < 3; ++r)
        out[r] = pc.P[r * 4 + 0] * Xw[0] + pc.P[r * 4 + 1] * Xw[1] + pc.P[r * 4 + 2] * Xw[2] + pc.P[r * 4 + 3];
}
}  // namespace orc

int orc_warp_from_depth(int V, int w, int h, int dsf, const float *depth, int depth_channels, const lfrv_camera *cams,
                        const lfrv_camera *target, int faithful, float *tau) {
    const size_t n = (size_t)w * h;
    const int W = target->width, H = target->height;
    const double kInvalid = 1000.0;
    std::vector<float> ud((size_t)W * H, (float)kInvalid);
    const orc::GlmCam u = orc::glm_cam(*target);
    for (int v = 0; v < V; ++v) {
        const orc::GlmCam c = orc::glm_cam(cams[v]);
        const float *dz = depth + (size_t)v * depth_channels * n;
        float *tv = tau + (size_t)v * 3 * n;
        for (size_t m = 0; m < n; ++m) {
            const float d = dz[m];
            if (d < 1.0 / kInvalid || kInvalid < d) {
                tv[m] = (float)-(double)w;
                tv[n + m] = tv[2 * n + m] = (float)-(double)h;
                continue;
            }
            const float x = (float)(m % w), y = (float)(m / w);
            float X[3];
            orc::wfd_transfer(c, c, u, d, x + 0.5f, y + 0.5f, X);
            const float txf = X[0] / X[2], tyf = X[1] / X[2];
            tv[m] = txf;
            tv[n + m] = tv[2 * n + m] = tyf;
            for (int i = 0; i < dsf; ++i)
                for (int j = 0; j < dsf; ++j) {
                    const int px = (int)txf - dsf / 2 + j, py = (int)tyf - dsf / 2 + i;
                    if (0 <= px && px <= W - 1 && 0 <= py && py <= H - 1) {
                        float &slot = ud[(size_t)py * W + px];
                        if (X[2] < slot) slot = X[2];
                    }
                }
        }
    }
    for (int v = 0; v < V; ++v) {
        const orc::GlmCam c = orc::glm_cam(cams[v]);
        const orc::GlmCam &rc = faithful ? c : u;
        float *tv = tau + (size_t)v * 3 * n;
        for (size_t m = 0; m < n; ++m) {
            const double tx = tv[m], ty = tv[n + m];
            float u_d = 0.f, u_norm = 0.f;
            for (int i = 0; i < dsf + 1; ++i)
                for (int j = 0; j < dsf + 1; ++j) {
                    const int px = (int)std::floor(tx - (double)(float)dsf * 0.5 + 0.5) + j;
                    const int py = (int)std::floor(ty - (double)(float)dsf * 0.5 + 0.5) + i;
                    if (!(0 <= px && px <= W - 1 && 0 <= py && py <= H - 1)) continue;
                    const float zu = ud[(size_t)py * W + px];
                    if (zu == (float)kInvalid) continue;
                    float dx = 1.0f, dy = 1.0f;
                    if (j == 0) dx = (float)(((double)(float)px + 0.5) - (tx - 0.5 * (double)(float)dsf));
                    else if (j == dsf) dx = (float)((tx + 0.5 * (double)(float)dsf) - ((double)(float)px - 0.5));
                    if (i == 0) dy = (float)(((double)(float)py + 0.5) - (ty - 0.5 * (double)(float)dsf));
                    else if (i == dsf) dy = (float)((ty + 0.5 * (double)(float)dsf) - ((double)(float)py - 0.5));
                    u_d += dx * dy * zu;
                    u_norm += dx * dy;
                }
            if (u_norm == 0.0f) {
                tv[m] = (float)-(double)w;
                tv[n + m] = tv[2 * n + m] = (float)-(double)h;
                continue;
            }
            u_d /= u_norm;
            float X[3];
            orc::wfd_transfer(u, rc, c, u_d, (float)((int)tx) + 0.5f, (float)((int)ty) + 0.5f, X);
            const int ox = (int)(X[0] / X[2]), oy = (int)(X[1] / X[2]);
            const int x = (int)(m % w), y = (int)(m / w);
            if (ox - x < -10 || 10 < ox - x || oy - y < -10 || 10 < oy - y) {
                tv[m] = (float)(-(double)w * 2.0);
                tv[n + m] = tv[2 * n + m] = (float)(-(double)h * 2.0);
            }
        }
    }
    return 0;
}

// fromRadial2Ortho.frag:10-23 (FrameBuffer::fromRadial2Ortho, sources/openGL/frameBuffer.cpp:263-300), in
// place on V x 3 x n depth maps (radial depth and its x / y derivatives): with X = K^-1 (x + 1/2, y + 1/2, 1)
// and d = |X|, z_o = z / d, dz_o/dx = dz/dx / d - z (X . K^-1 column 0) / d^3, and likewise for y with column 1.
// The shader's pow(d, 3.0) is written d * d * d here.
int orc_depth_radial_to_ortho(int V, int w, int h, const lfrv_camera *cams, float *depth) {
    const size_t n = (size_t)w * h;
    for (int v = 0; v < V; ++v) {
        const orc::Cam c = orc::to_cam(cams[v]);
        float *dz = depth + (size_t)v * 3 * n;
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const size_t m = (size_t)y * w + x;
                const double px = x + 0.5, py = y + 0.5;
                const double X[3] = {c.Kinv[0] * px + c.Kinv[1] * py + c.Kinv[2],
                                     c.Kinv[3] * px + c.Kinv[4] * py + c.Kinv[5],
                                     c.Kinv[6] * px + c.Kinv[7] * py + c.Kinv[8]};
                const double d = std::sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]), d3 = d * d * d;
                const double c0 = X[0] * c.Kinv[0] + X[1] * c.Kinv[3] + X[2] * c.Kinv[6];  // X . column 0
                const double c1 = X[0] * c.Kinv[1] + X[1] * c.Kinv[4] + X[2] * c.Kinv[7];  // X . column 1
                const double z = dz[m], zx = dz[n + m], zy = dz[2 * n + m];
                dz[m] = (float)(z / d);
                dz[n + m] = (float)(zx / d - z * c0 / d3);
                dz[2 * n + m] = (float)(zy / d - z * c1 / d3);
            }
    }
    return 0;
}

// Footprint weights of one source pixel (for the kernel pinning tests).
int orc_footprint(int prec, float tx, float ty, int dsf, int W, int H, int *x0, int *y0, float *A) {
    if (prec == 0) {
        orc::Footprint<double> fp;
        orc::footprint<double>(tx, ty, dsf, W, H, fp);
        *x0 = fp.x0;
        *y0 = fp.y0;
        for (int e = 0; e < fp.ks * fp.ks; ++e) A[e] = (float)fp.A[e];
    } else {
        orc::Footprint<float> fp;
        orc::footprint<float>(tx, ty, dsf, W, H, fp);
        *x0 = fp.x0;
        *y0 = fp.y0;
        for (int e = 0; e < fp.ks * fp.ks; ++e) A[e] = fp.A[e];
    }
    return 0;
}

int orc_gaussian_blur(int prec, int W, int H, const float *in, float *out) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        std::vector<T> i = conv<T>(in, (size_t)W * H), o((size_t)W * H);
        orc::gaussian_blur<T>(W, H, i.data(), o.data());
        back(o, out);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

int orc_sobel(int prec, int W, int H, const float *rgb, const uint8_t *vis, float *gx, float *gy) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        const size_t N = (size_t)W * H;
        std::vector<T> c = conv<T>(rgb, 3 * N), a = conv<T>(gx, N), b = conv<T>(gy, N);
        orc::sobel<T>(W, H, c.data(), c.data() + N, c.data() + 2 * N, a.data(), b.data(), vis);
        back(a, gx);
        back(b, gy);
        return 0;
    };
    return prec == 0 ? run(double()) : run(float());
}

}  // extern "C"
