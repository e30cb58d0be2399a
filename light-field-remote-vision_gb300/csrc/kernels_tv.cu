// kernels_tv.cu -- corrected IBR_color: the weighted TV_F objective solved to a certified primal-dual gap.
//
// No reference counterpart. The reference's ISTA step (sources/optimization.cu:1751-1832) normalises the data
// term's gradient by the coverage and clamps it, and reports an energy that is not its objective; in corrected mode
// the library minimises
//   E(u) = f(u) + lambda J_g(u) over [0, 1]^{3N},
//   f(u) = alpha sigma^2 / 2 sum_i sum_{m in S_i} w_im |A_i u - v_i|^2_m        (S_i: view i's splat set),
//   J_g(u) = sum_x g_x |grad u(x)|_F                                           (the TV_F of vtv_rof.cu:280-320),
// by FISTA in the diagonal metric D = max(alpha sigma^2 sum_i A_i^T w_i, 1) (a majoriser of f's Hessian: the rows
// of A_i sum to 1), each step a weighted ROF problem solved by the fast gradient projection (FGP) on its dual, and
// certifies E(u) - E* <= lambda sum_x [g_x |grad u|_F - <grad u, p>] + sum [u c - min(0, c)], c = grad f(u) -
// lambda div p. The host loop is color_solve_tv (host.cpp); the CPU restatement is oracle tv_solve.
#include "device_common.cuh"
#include "kernels.h"
#include "lfrv_internal.h"

#include <mutex>
#include <type_traits>

namespace lfrv {

constexpr float kTvDelta = 1.0f;  // floor of the metric D (pixels without data keep a proximal term)

// ------------------------------------------------------------------ per-pixel set-up
template <int KS>
__global__ void k_tv_metric(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                            const unsigned int *__restrict__ entries, const float *__restrict__ tau,
                            const float *__restrict__ wgt, float as2, float lambda, float *__restrict__ D,
                            float *__restrict__ lam) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const SplatSrc src{{wgt, wgt, wgt}, {(size_t)n, (size_t)n, (size_t)n}, nullptr};
    float acc[3], norm;
    splat_accumulate<KS, 1>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    const size_t o = (size_t)y * W + x;
    const float d = fmaxf(as2 * acc[0], kTvDelta);
    D[o] = d;
    lam[o] = lambda / d;
}

// Dual step 1 / L_x, L_x = 8 max(lam_x, lam_{x+1}, lam_{x+W}): the dual Hessian grad diag(lam) grad^T is at most
// diag(L) (each dual entry enters the divergence at two pixels, each divergence has four terms).
__global__ void k_tv_linv(int W, int H, const float *__restrict__ lam, float *__restrict__ linv) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t o = (size_t)y * W + x;
    float m = lam[o];
    if (x < W - 1) m = fmaxf(m, lam[o + 1]);
    if (y < H - 1) m = fmaxf(m, lam[o + W]);
    linv[o] = 1.0f / (8.0f * m);
}

template <int KS>
__global__ void k_tv_gradf(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                           const unsigned int *__restrict__ entries, const float *__restrict__ tau,
                           const float *__restrict__ res, float as2, float *__restrict__ gf) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t s3 = (size_t)3 * n;
    const SplatSrc src{{res, res + n, res + 2 * (size_t)n}, {s3, s3, s3}, nullptr};
    float acc[3], norm;
    splat_accumulate<KS, 3>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    const size_t o = (size_t)y * W + x, N = (size_t)W * H;
#pragma unroll
    for (int c = 0; c < 3; ++c) gf[c * N + o] = as2 * acc[c];
}

// div of a dual field at (x, y): the negative adjoint of the forward gradient with zero at the last column / row.
template <typename TD>
__device__ __forceinline__ TD tv_div(const TD *px, const TD *py, int W, int H, int x, int y, size_t o) {
    TD d = 0;
    if (x < W - 1) d += px[o];
    if (x > 0) d -= px[o - 1];
    if (y < H - 1) d += py[o];
    if (y > 0) d -= py[o - W];
    return d;
}

// ------------------------------------------------------------------ certificate
// One-dimensional blocks of kGapBX * kGapBY threads (block_sum indexes warps by threadIdx.x), each covering a
// kGapBX x kGapBY patch of pixels.
constexpr int kGapBX = 32, kGapBY = 8;
__global__ void __launch_bounds__(kGapBX * kGapBY) k_tv_gap(int W, int H, const float *__restrict__ u,
                                                            const float *__restrict__ gf, const double *__restrict__ P,
                                                            const float *__restrict__ g, float lambda,
                                                            double *__restrict__ partial) {
    __shared__ double red[kGapBX * kGapBY / 32];
    const int x = blockIdx.x * kGapBX + (int)(threadIdx.x % kGapBX);
    const int y = blockIdx.y * kGapBY + (int)(threadIdx.x / kGapBX);
    const size_t N = (size_t)W * H;
    double tv = 0.0, inner = 0.0, box = 0.0;
    if (x < W && y < H) {
        const size_t o = (size_t)y * W + x;
        double n2 = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float *uc = u + c * N;
            const double gxv = x < W - 1 ? (double)uc[o + 1] - (double)uc[o] : 0.0;
            const double gyv = y < H - 1 ? (double)uc[o + W] - (double)uc[o] : 0.0;
            n2 += gxv * gxv + gyv * gyv;
            const double *px = P + c * N, *py = P + (3 + c) * N;
            inner += gxv * px[o] + gyv * py[o];
            const double cc = (double)gf[c * N + o] - (double)lambda * tv_div(px, py, W, H, x, y, o);
            box += (double)uc[o] * cc - fmin(0.0, cc);
        }
        tv = (double)g[o] * sqrt(n2);
    }
    const int b = blockIdx.y * gridDim.x + blockIdx.x, nb = gridDim.x * gridDim.y;
    const double s0 = block_sum<kGapBX * kGapBY>(tv, red);
    if (threadIdx.x == 0) partial[b] = s0;
    const double s1 = block_sum<kGapBX * kGapBY>(inner, red);
    if (threadIdx.x == 0) partial[nb + b] = s1;
    const double s2 = block_sum<kGapBX * kGapBY>(box, red);
    if (threadIdx.x == 0) partial[2 * nb + b] = s2;
}

__global__ void k_tv_fstep(size_t N, const float *__restrict__ u, const float *__restrict__ up,
                           const float *__restrict__ gf, const float *__restrict__ gfp, const float *__restrict__ D,
                           float theta_arg, const TvLoopState *__restrict__ loop, float *__restrict__ F) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * N) return;
    const float theta = loop ? loop->theta : theta_arg;
    const float y = u[i] + theta * (u[i] - up[i]);
    const float gy = (1.0f + theta) * gf[i] - theta * gfp[i];
    F[i] = y - gy / D[i % N];
}

__global__ void k_tv_clamp(size_t n, const float *__restrict__ in, float *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = fminf(1.0f, fmaxf(0.0f, in[i]));
}

// ------------------------------------------------------------------ FGP on the weighted ROF dual
// One cooperative launch runs every inner iteration. Temporally blocked: a block takes a tile and a halo of K
// pixels and runs K iterations on that region before it writes the tile back and the grid synchronises (each
// iteration's dependence reaches one pixel in each direction, diagonals included, so the tile stays exact; the
// updated part of the region shrinks by a pixel per iteration to what the tile still depends on). Per iteration:
//   u = clamp(F + lam div q, 0, 1);  p' = proj_{|.|_F <= g}(q + grad u / L);  q = p' + beta_j (p' - p);  p = p'
// with beta_j = (s_j - 1) / s_{j+1}, s_0 = 1, s_{j+1} = (1 + sqrt(1 + 4 s_j^2)) / 2 (Beck and Teboulle's FGP).
// Every thread owns the same PPT region pixels throughout: their q, p, F, lam, 1/L and g stay in registers, and
// shared memory carries what the neighbours read (u for the gradient, the x and y components of q for the
// divergence). The block sizes split the region evenly.
// The dual p and the momentum point q are stored in FP64 (12 planes); u, F, lam, 1/L and g are FP32. TD is the
// dual's arithmetic type. In FP32 the dual's rounding (a few ulp of |p| <= g) leaves lambda div p, and with it the
// certificate's box term, a noise floor near 4e-4 relative at 256^2; with the double-float type below (about 44
// bits) the certificate reaches 1e-4, as with FP64 (the oracle's FP32 mirror shows the floor, its FP64 dual does
// not). FP64 arithmetic is slow on this GPU's narrow FP64 pipe and double-float costs several FP32 operations per
// operation, so the host runs TD = float while the gap is far above its floor and TD = dfloat to finish.
// Double-float arithmetic (an unevaluated sum hi + lo of two floats, about 44 significant bits): the dual's
// arithmetic where FP32 would leave its noise floor, on the FP32 pipes. Sums use the error-free two-sum (Knuth)
// and products the FMA-based two-product (Dekker's splitting replaced by fmaf), each renormalised with the
// fast two-sum; the add is the accurate form (both parts' errors carried), since p' - p cancels.
struct dfloat {
    float hi, lo;
    __device__ __forceinline__ dfloat() : hi(0.f), lo(0.f) {}
    __device__ __forceinline__ dfloat(int v) : hi((float)v), lo(0.f) {}
    __device__ __forceinline__ dfloat(float v) : hi(v), lo(0.f) {}
    __device__ __forceinline__ dfloat(double v) {
        hi = __double2float_rn(v);
        lo = __double2float_rn(v - (double)hi);
    }
    __device__ __forceinline__ dfloat(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit operator float() const { return hi + lo; }
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return dfloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return dfloat(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
    dfloat s = df_two_sum(a.hi, b.hi);
    const dfloat t = df_two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = df_fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat &operator-=(dfloat &a, dfloat b) { return a = a - b; }
__device__ __forceinline__ bool operator>(dfloat a, dfloat b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
// a + b for a float b (no cancellation concerns: one two-sum, the low part added, renormalised)
__device__ __forceinline__ dfloat df_add_f(dfloat a, float b) {
    const dfloat s = df_two_sum(a.hi, b);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
// a + b where the sum cannot cancel (both of one sign, or b much smaller): the low parts are added in float
__device__ __forceinline__ dfloat df_add_sloppy(dfloat a, dfloat b) {
    const dfloat s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
// a0 - a1 + a2 - a3 rounded to float: the high parts' sums are exact (two-sum), their errors and the low parts
// are added in float, so the result carries an error of about one float ulp of itself (not of the terms)
__device__ __forceinline__ float df_div4(dfloat a0, dfloat a1, dfloat a2, dfloat a3) {
    const dfloat h1 = df_two_sum(a0.hi, -a1.hi), h2 = df_two_sum(a2.hi, -a3.hi), h = df_two_sum(h1.hi, h2.hi);
    const float lo = __fadd_rn(__fsub_rn(a0.lo, a1.lo), __fsub_rn(a2.lo, a3.lo));
    return __fadd_rn(h.hi, __fadd_rn(__fadd_rn(__fadd_rn(h1.lo, h2.lo), h.lo), lo));
}

constexpr int kFgpTX = 32, kFgpTY = 16;
template <int K>
constexpr int fgp_rn() { return (kFgpTX + 2 * K) * (kFgpTY + 2 * K); }
template <typename TD, int K>
constexpr size_t fgp_smem() { return (size_t)6 * fgp_rn<K>() * sizeof(TD) + (size_t)3 * fgp_rn<K>() * sizeof(float); }
constexpr int kFgpBetaTable = 256;

template <typename TD, int K, int THREADS>
__global__ void __launch_bounds__(THREADS) k_tv_fgp(int W, int H, int niter, const float *__restrict__ F,
                                                    const float *__restrict__ lam, const float *__restrict__ linv,
                                                    const float *__restrict__ g, double *P0, double *P1, double *Q0,
                                                    double *Q1, float *__restrict__ U, GridBarrier gb) {
    constexpr int RX = kFgpTX + 2 * K, RY = kFgpTY + 2 * K, RN = RX * RY;
    constexpr int PPT = (RN + THREADS - 1) / THREADS;
    constexpr unsigned kIn = 1, kFx = 2, kFy = 4, kBx = 8, kBy = 16, kTile = 32, kRx = 64, kRy = 128;
    constexpr int kDistShift = 8;
    extern __shared__ __align__(16) unsigned char fgp_sm[];
    TD *sQx = reinterpret_cast<TD *>(fgp_sm), *sQy = sQx + 3 * RN;
    float *sU = reinterpret_cast<float *>(sQy + 3 * RN);
    // the momentum weights beta_j of the first kFgpBetaTable iterations, worked out once per block (the FP64
    // square root and division are long sequences on this GPU's narrow FP64 pipe; later iterations, if any,
    // continue the sequence inline)
    __shared__ double s_beta[kFgpBetaTable];
    __shared__ double s_tail;  // s_j after the table
    if (threadIdx.x == 0) {
        double sj = 1.0;
        for (int j = 0; j < min(niter, kFgpBetaTable); ++j) {
            const double s1 = 0.5 * (1.0 + sqrt(1.0 + 4.0 * sj * sj));
            s_beta[j] = (sj - 1.0) / s1;
            sj = s1;
        }
        s_tail = sj;
    }
    __syncthreads();
    const int tiles_x = (W + kFgpTX - 1) / kFgpTX, ntiles = tiles_x * ((H + kFgpTY - 1) / kFgpTY);
    const size_t N = (size_t)W * H;
    unsigned int gen = 0;
    double s_step = s_tail;  // s_j of the first iteration past the table (every thread follows the same sequence)
    int step = 0;
    for (int done = 0; done < niter; done += K, ++step) {
        const int iters = min(K, niter - done);
        const double *Pi = (step & 1) ? P1 : P0;
        double *Po = (step & 1) ? P0 : P1;
        const double *Qi = step == 0 ? P0 : ((step & 1) ? Q1 : Q0);  // q starts at p
        double *Qo = (step & 1) ? Q0 : Q1;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int rx0 = (t % tiles_x) * kFgpTX - K, ry0 = (t / tiles_x) * kFgpTY - K;
            TD q[PPT][6], p[PPT][6];
            float f[PPT][3], lm[PPT], li[PPT], gg[PPT];
            unsigned int fl[PPT];
            size_t go[PPT];
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                const int i = threadIdx.x + k * THREADS;
                const int lx = i % RX, ly = i / RX, gx = rx0 + lx, gy = ry0 + ly;
                const bool in = i < RN && gx >= 0 && gx < W && gy >= 0 && gy < H;
                unsigned int f0 = 0;
                if (in) {
                    f0 |= kIn;
                    if (gx < W - 1) f0 |= kFx;
                    if (gy < H - 1) f0 |= kFy;
                    if (gx > 0) f0 |= kBx;
                    if (gy > 0) f0 |= kBy;
                    if (lx + 1 < RX) f0 |= kRx;
                    if (ly + 1 < RY) f0 |= kRy;
                    if (lx >= K && lx < K + kFgpTX && ly >= K && ly < K + kFgpTY) f0 |= kTile;
                    const int dx = max(max(K - lx, lx - (K + kFgpTX - 1)), 0);
                    const int dy = max(max(K - ly, ly - (K + kFgpTY - 1)), 0);
                    f0 |= (unsigned int)max(dx, dy) << kDistShift;
                }
                fl[k] = f0;
                const size_t o = in ? (size_t)gy * W + gx : 0;
                go[k] = o;
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    q[k][c] = in ? (TD)__ldcg(Qi + c * N + o) : TD(0);
                    p[k][c] = in ? (TD)__ldcg(Pi + c * N + o) : TD(0);
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) f[k][c] = in ? __ldg(F + c * N + o) : 0.f;
                lm[k] = in ? __ldg(lam + o) : 0.f;
                li[k] = in ? __ldg(linv + o) : 0.f;
                gg[k] = in ? __ldg(g + o) : 0.f;
                if (i < RN) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        sQx[c * RN + i] = q[k][c];
                        sQy[c * RN + i] = q[k][3 + c];
                    }
                }
            }
            __syncthreads();
            double s = s_step;
            for (int it = 0; it < iters; ++it) {
                const int j = done + it;
                double s1 = s;
                TD beta;
                if (j < kFgpBetaTable) {
                    beta = (TD)s_beta[j];
                } else {
                    s1 = 0.5 * (1.0 + sqrt(1.0 + 4.0 * s * s));
                    beta = (TD)((s - 1.0) / s1);
                }
                // u(q) where the tile still depends on it (values next to the region's edge are stale and stay
                // outside the tile)
                const unsigned int u_reach = (unsigned int)(iters - it) << kDistShift;
                const unsigned int p_reach = (unsigned int)(iters - it - 1) << kDistShift;
#pragma unroll
                for (int k = 0; k < PPT; ++k) {
                    if (!(fl[k] & kIn) || (fl[k] & ~0xFFu) > u_reach) continue;
                    const int i = threadIdx.x + k * THREADS;
                    const int lx = i % RX, ly = i / RX;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        float dv;
                        if constexpr (std::is_same<TD, dfloat>::value) {
                            const dfloat z;
                            dv = df_div4((fl[k] & kFx) ? q[k][c] : z,
                                         ((fl[k] & kBx) && lx > 0) ? sQx[c * RN + i - 1] : z,
                                         (fl[k] & kFy) ? q[k][3 + c] : z,
                                         ((fl[k] & kBy) && ly > 0) ? sQy[c * RN + i - RX] : z);
                        } else {
                            TD d = 0;
                            if (fl[k] & kFx) d += q[k][c];
                            if (fl[k] & kBx) d -= lx > 0 ? sQx[c * RN + i - 1] : TD(0);
                            if (fl[k] & kFy) d += q[k][3 + c];
                            if (fl[k] & kBy) d -= ly > 0 ? sQy[c * RN + i - RX] : TD(0);
                            dv = (float)d;
                        }
                        sU[c * RN + i] = fminf(1.0f, fmaxf(0.0f, f[k][c] + lm[k] * dv));
                    }
                }
                __syncthreads();
                // p' = proj(q + grad u / L), q = p' + beta (p' - p) (own pixel)
#pragma unroll
                for (int k = 0; k < PPT; ++k) {
                    if (!(fl[k] & kIn) || (fl[k] & ~0xFFu) > p_reach) continue;
                    const int i = threadIdx.x + k * THREADS;
                    TD v[6];
                    TD n2 = 0;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float *uc = sU + c * RN;
                        const float ui = uc[i];
                        const float ur = (fl[k] & kRx) ? uc[i + 1] : 0.f;
                        const float ud = (fl[k] & kRy) ? uc[i + RX] : 0.f;
                        const float gxv = (fl[k] & kFx) ? ur - ui : 0.f;
                        const float gyv = (fl[k] & kFy) ? ud - ui : 0.f;
                        if constexpr (std::is_same<TD, dfloat>::value) {
                            v[c] = df_add_f(q[k][c], gxv * li[k]);
                            v[3 + c] = df_add_f(q[k][3 + c], gyv * li[k]);
                            n2 = df_add_sloppy(df_add_sloppy(n2, v[c] * v[c]), v[3 + c] * v[3 + c]);
                        } else {
                            v[c] = q[k][c] + (TD)(gxv * li[k]);
                            v[3 + c] = q[k][3 + c] + (TD)(gyv * li[k]);
                            n2 += v[c] * v[c] + v[3 + c] * v[3 + c];
                        }
                    }
                    // projection onto |p| <= g without a square root or division in the extended type: r = 1 / sqrt(n2)
                    // from the FP32 estimate and two Newton steps in TD (relative error ~1e-13 in double-float),
                    // applied only where the ball constraint is active
                    const TD gv = (TD)gg[k];
                    TD sc = 1;
                    if (n2 > gv * gv) {
                        TD r = (TD)rsqrtf((float)n2);
                        if (sizeof(TD) == sizeof(double)) {
                            r = r * (TD(1.5) - TD(0.5) * n2 * r * r);
                            r = r * (TD(1.5) - TD(0.5) * n2 * r * r);
                        }
                        sc = gv * r;
                    }
#pragma unroll
                    for (int c = 0; c < 6; ++c) {
                        const TD pn = v[c] * sc;
                        if constexpr (std::is_same<TD, dfloat>::value) q[k][c] = df_add_sloppy(pn, beta * (pn - p[k][c]));
                        else q[k][c] = pn + beta * (pn - p[k][c]);
                        p[k][c] = pn;
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        sQx[c * RN + i] = q[k][c];
                        sQy[c * RN + i] = q[k][3 + c];
                    }
                }
                __syncthreads();
                s = s1;
            }
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                if ((fl[k] & (kIn | kTile)) != (kIn | kTile)) continue;
                const size_t o = go[k];
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    Po[c * N + o] = (double)p[k][c];
                    Qo[c * N + o] = (double)q[k][c];
                }
            }
            __syncthreads();  // the next tile overwrites the staged region
        }
        for (int it = 0; it < iters; ++it)
            if (done + it >= kFgpBetaTable) s_step = 0.5 * (1.0 + sqrt(1.0 + 4.0 * s_step * s_step));
        if (!grid_sync(gb, gen)) return;
    }
    // the final dual sits in P0 after an even number of super-steps, else in P1; u = clamp(F + lam div p)
    const int steps = (niter + K - 1) / K;
    const double *Pf = (steps & 1) ? P1 : P0;
    double *Pother = (steps & 1) ? P0 : P1;
    for (size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x; o < N; o += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(o % W), y = (int)(o / W);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double d = tv_div(Pf + c * N, Pf + (3 + c) * N, W, H, x, y, o);
            U[c * N + o] = fminf(1.0f, fmaxf(0.0f, F[c * N + o] + lam[o] * (float)d));
        }
    }
    // the caller keeps its dual in P0: copy it there when the last super-step wrote P1
    if (steps & 1) {
        if (!grid_sync(gb, gen)) return;  // every block has read P1's neighbours above
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < 6 * N; i += (size_t)gridDim.x * blockDim.x)
            Pother[i] = Pf[i];
    }
}

// ------------------------------------------------------------------ launchers
static inline dim3 tv_grid(int W, int H, dim3 b) { return dim3((W + b.x - 1) / b.x, (H + b.y - 1) / b.y); }

void launch_tv_metric(const Geometry &G, const Buckets &B, const float *tau, const float *wgt, float as2, float lambda,
                      float *D, float *lam, float *linv, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "tv_metric", st);
    const dim3 b(32, 8), g = tv_grid(G.W, G.H, b);
    LFRV_KS_DISPATCH(G.dsf + 1, k_tv_metric, g, b, st, G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries, tau, wgt,
                     as2, lambda, D, lam);
    k_tv_linv<<<g, b, 0, st>>>(G.W, G.H, lam, linv);
    lc.add(2);
}

void launch_tv_gradf(const Geometry &G, const Buckets &B, const float *tau, const float *res, float as2, float *gf,
                     cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "tv_gradf", st);
    const dim3 b(32, 8), g = tv_grid(G.W, G.H, b);
    LFRV_KS_DISPATCH(G.dsf + 1, k_tv_gradf, g, b, st, G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries, tau, res, as2,
                     gf);
    lc.add(1);
}

int tv_gap_partials(int W, int H) { return ((W + kGapBX - 1) / kGapBX) * ((H + kGapBY - 1) / kGapBY); }

void launch_tv_gap(int W, int H, const float *u, const float *gf, const double *P, const float *g, float lambda,
                   double *partial, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "tv_gap", st);
    const dim3 gr = tv_grid(W, H, dim3(kGapBX, kGapBY));
    k_tv_gap<<<gr, kGapBX * kGapBY, 0, st>>>(W, H, u, gf, P, g, lambda, partial);
    lc.add(1);
}

void launch_tv_fstep(int W, int H, const float *u, const float *up, const float *gf, const float *gfp, const float *D,
                     float theta, float *F, cudaStream_t st, LaunchCounter &lc, const TvLoopState *loop) {
    ProfScope _ps(lc, "tv_fstep", st);
    const size_t N = (size_t)W * H;
    k_tv_fstep<<<(unsigned)((3 * N + 255) / 256), 256, 0, st>>>(N, u, up, gf, gfp, D, theta, loop, F);
    lc.add(1);
}

// The stop test and momentum update of the corrected IBR_color solve on the device (TvSolve::decide and the scalar
// part of TvSolve::step, the same double arithmetic), for a solve whose loop runs as a conditional graph: one
// thread reads the certificate sums, records the energy, decides, and sets the loop's and the arithmetic's
// conditions.
__global__ void k_tv_decide(const double *__restrict__ sums, double dt_alpha, double lambda, double tol, int niter,
                            double extended_below, TvLoopState *loop, double *trace, int trace_cap,
                            cudaGraphConditionalHandle h_loop, cudaGraphConditionalHandle h_extended) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double f = 0.5 * dt_alpha * sums[1];
    const double E = f + lambda * sums[4];
    const double gap_abs = lambda * (sums[4] - sums[5]) + sums[6];
    const double gap = E > 0 ? gap_abs / E : 1e300;
    if (trace && loop->trace_pos < trace_cap) trace[loop->trace_pos++] = E;
    bool done = loop->k >= niter || (tol > 0 && gap <= tol);
    if (!isfinite(E) || !isfinite(gap)) {
        loop->err = 1;
        done = true;
    }
    loop->E = E;
    loop->gap = gap;
    if (!done) {
        if (E > loop->E_prev) loop->t = 1.0;  // function-value restart of the momentum
        loop->E_prev = E;
        const double t = loop->t, t1 = 0.5 * (1.0 + sqrt(1.0 + 4.0 * t * t));
        loop->theta = (float)((t - 1.0) / t1);
        loop->t = t1;
        loop->extended = loop->extended || gap < extended_below;
        loop->k += 1;
    }
    loop->done = done ? 1 : 0;
    cudaGraphSetConditional(h_loop, done ? 0u : 1u);
    cudaGraphSetConditional(h_extended, loop->extended ? 1u : 0u);
}

void launch_tv_decide(const double *sums, double dt_alpha, double lambda, double tol, int niter, TvLoopState *loop,
                      double *trace, int trace_cap, cudaGraphConditionalHandle h_loop,
                      cudaGraphConditionalHandle h_extended, cudaStream_t st, LaunchCounter &lc) {
    k_tv_decide<<<1, 32, 0, st>>>(sums, dt_alpha, lambda, tol, niter, kTvExtendedBelow, loop, trace, trace_cap, h_loop,
                                  h_extended);
    lc.add(1);
}

void launch_tv_clamp(size_t n, const float *in, float *out, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "tv_clamp", st);
    k_tv_clamp<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, in, out);
    lc.add(1);
}

// Instantiations the FGP autotuner chooses from, per arithmetic: (iterations per super-step K, threads); the
// region of K = 2, 4, 6, 8 holds 720, 960, 1232, 1536 pixels, two per thread. All give the same iterates.
struct FgpVariant {
    int K, threads;
    const void *kernel;
    size_t smem;
};
static const FgpVariant kFgpFloat[] = {
    {4, 480, (const void *)k_tv_fgp<float, 4, 480>, fgp_smem<float, 4>()},
    {6, 640, (const void *)k_tv_fgp<float, 6, 640>, fgp_smem<float, 6>()},
    {8, 768, (const void *)k_tv_fgp<float, 8, 768>, fgp_smem<float, 8>()},
};
static const FgpVariant kFgpDfloat[] = {
    {2, 384, (const void *)k_tv_fgp<dfloat, 2, 384>, fgp_smem<dfloat, 2>()},
    {4, 480, (const void *)k_tv_fgp<dfloat, 4, 480>, fgp_smem<dfloat, 4>()},
};
int tv_fgp_variant_count(bool extended) { return extended ? 2 : 3; }
int tv_fgp_default_variant(bool extended) { return extended ? 1 : 2; }

cudaError_t launch_tv_fgp(int W, int H, int niter, const float *F, const float *lam, const float *linv, const float *g,
                          double *P0, double *P1, double *Q0, double *Q1, float *U, GridBarrier gb, cudaStream_t st,
                          LaunchCounter &lc, bool extended, int variant) {
    ProfScope _ps(lc, extended ? "tv_fgp_df" : "tv_fgp", st);
    if (variant < 0 || variant >= tv_fgp_variant_count(extended)) variant = tv_fgp_default_variant(extended);
    const FgpVariant &R = extended ? kFgpDfloat[variant] : kFgpFloat[variant];
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    static std::mutex mu;
    static bool attr_set[64] = {};
    if (dev >= 0 && dev < 64) {
        std::lock_guard<std::mutex> lock(mu);
        if (!attr_set[dev]) {
            for (const FgpVariant &v : kFgpFloat)
                cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v.smem);
            for (const FgpVariant &v : kFgpDfloat)
                cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v.smem);
            attr_set[dev] = true;
        }
    }
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, R.kernel, R.threads, R.smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int ntiles = ((W + kFgpTX - 1) / kFgpTX) * ((H + kFgpTY - 1) / kFgpTY);
    const int resident = sms * per_sm;
    // as few blocks as keep the per-block tile count at its minimum (no block waits for a straggler's extra tile)
    const int per_block = (ntiles + resident - 1) / resident;
    const int blocks = std::max(1, (ntiles + per_block - 1) / per_block);
    void *args[] = {&W, &H, &niter, (void *)&F, (void *)&lam, (void *)&linv, (void *)&g, &P0, &P1, &Q0, &Q1, &U, &gb};
    lc.add(1);
    return cudaLaunchCooperativeKernel(R.kernel, dim3(blocks), dim3(R.threads), args, R.smem, st);
}

}  // namespace lfrv
