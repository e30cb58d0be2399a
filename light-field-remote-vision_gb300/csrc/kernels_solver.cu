// kernels_solver.cu -- solver-stage kernels of the IBR_color / IBR_gradient path (sm_103a).
//
// Layout in HBM (all planar float32, row-major, top-left origin):
//   per view v (V views, n = w*h source pixels): img[v][3][n], tau[v][2][n] (tau_x, tau_y),
//     dp[v][2][n] (sigma_z * dtau/dz), wgt[v][n] (omega_i), res[v][3][n] (weighted residual scratch)
//   target (N = W*H pixels): U[3][N], P[6][N] duals (px0,py0,px1,py1,px2,py2), F[3][N], g[N], masks.
//
// The reference splats A_i^T r with one launch per host-computed non-overlapping cell segment
// (sources/optimization.cu:882-1025, 1921-1951). Here the scatter becomes a deterministic gather: source
// pixels of all views are bucketed by the anchor of their footprint (counting sort, buckets sorted by
// (view, pixel)), and every target pixel reads the ks x ks anchor buckets that can reach it, recomputing
// the footprint weights from tau instead of storing A (the reference stores ks^2 floats per source pixel).
#include <algorithm>
#include <mutex>

#include <cuda_bf16.h>

#include "device_common.cuh"
#include "kernels.h"

namespace lfrv {

// Storage of the per-view stacks: FP32, or BF16 when the configuration asks for it (loads widen to FP32, and
// every accumulation stays FP32).
__device__ __forceinline__ float ldv(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ldv(const __nv_bfloat16 *p) { return __bfloat162float(__ldg(p)); }
__device__ __forceinline__ void stv(float *p, float v) { *p = v; }
__device__ __forceinline__ void stv(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }


// ====================================================================== inverse footprint map
// Count and fill take kBucketPer source pixels per thread (m, m + blockDim.x, ...): each stage's loads and atomics
// for all of them are issued before any result is used, so their round trips to L2 overlap. Bucket of a
// splatted source pixel: its footprint anchor, offset by ks - 1 (-1: not splatted).
// The count also sets bit v of its bucket's view mask (ceil(V / 64) 64-bit words per bucket, word-major). A bucket
// whose count equals the mask's population holds one entry per view, and the entry of view v goes to slot
// popc(mask & (2^v - 1)): already in (view, pixel) order, with no atomic in the fill and nothing for the sort to
// do. Only buckets with two entries of one view take slots from the cursor (in arrival order) and need the sort.
constexpr int kBucketPer = 4;


__global__ void k_bucket_count(int V, int n, int W, int H, int dsf, int BW, const float *__restrict__ tau,
                               unsigned int *__restrict__ cnt, unsigned long long *__restrict__ mask, int nb) {
    const int v = (int)(blockIdx.x % (unsigned)V);
    const int m0 = (int)(blockIdx.x / (unsigned)V) * blockDim.x * kBucketPer + threadIdx.x;
    const float *tv = tau + (size_t)v * 2 * n;
    float tx[kBucketPer], ty[kBucketPer];
#pragma unroll
    for (int j = 0; j < kBucketPer; ++j) {
        const int m = min(m0 + j * (int)blockDim.x, n - 1);
        tx[j] = tv[m];
        ty[j] = tv[n + m];
    }
#pragma unroll
    for (int j = 0; j < kBucketPer; ++j) {
        const long long b = bucket_of(tx[j], ty[j], W, H, dsf, BW);
        if (m0 + j * (int)blockDim.x < n && b >= 0) {
            atomicAdd(&cnt[b], 1u);
            if (mask) atomicOr(&mask[(size_t)(v >> 6) * nb + b], 1ull << (v & 63));
        }
    }
}

// Views in bucket b's mask (mw words).
__device__ __forceinline__ unsigned int mask_pop(const unsigned long long *mask, int mw, int nb, long long b) {
    unsigned int c = 0;
    for (int w = 0; w < mw; ++w) c += (unsigned int)__popcll(mask[(size_t)w * nb + b]);
    return c;
}

// Whether bucket b's entries must come from the cursor and be sorted (see above).
__device__ __forceinline__ bool bucket_dup(const unsigned int *start, const unsigned long long *mask, int mw, int nb,
                                           long long b) {
    return !mask || start[b + 1] - start[b] != mask_pop(mask, mw, nb, b);
}

__global__ void k_bucket_fill(int V, int n, int W, int H, int dsf, int BW, const float *__restrict__ tau,
                              const unsigned int *__restrict__ start, unsigned int *__restrict__ cursor,
                              const unsigned long long *__restrict__ mask, int mw, int nb,
                              unsigned int *__restrict__ entries) {
    pdl_wait();
    pdl_trigger();
    const int v = (int)(blockIdx.x % (unsigned)V);
    const int m0 = (int)(blockIdx.x / (unsigned)V) * blockDim.x * kBucketPer + threadIdx.x;
    const float *tv = tau + (size_t)v * 2 * n;
    float tx[kBucketPer], ty[kBucketPer];
#pragma unroll
    for (int j = 0; j < kBucketPer; ++j) {
        const int m = min(m0 + j * (int)blockDim.x, n - 1);
        tx[j] = tv[m];
        ty[j] = tv[n + m];
    }
    long long b[kBucketPer];
    unsigned int slot[kBucketPer], base[kBucketPer];
#pragma unroll
    for (int j = 0; j < kBucketPer; ++j) {
        b[j] = m0 + j * (int)blockDim.x < n ? bucket_of(tx[j], ty[j], W, H, dsf, BW) : -1;
        slot[j] = 0u;
        base[j] = 0u;
        if (b[j] >= 0) {
            base[j] = start[b[j]];
            if (bucket_dup(start, mask, mw, nb, b[j])) {
                slot[j] = atomicAdd(&cursor[b[j]], 1u);
            } else {
                unsigned int below = 0;  // views before v in this bucket
                for (int w = 0; w < (v >> 6); ++w) below += (unsigned int)__popcll(mask[(size_t)w * nb + b[j]]);
                slot[j] = below + (unsigned int)__popcll(mask[(size_t)(v >> 6) * nb + b[j]] & ((1ull << (v & 63)) - 1ull));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kBucketPer; ++j)
        if (b[j] >= 0) entries[base[j] + slot[j]] = ((unsigned int)v << 24) | (unsigned int)(m0 + j * (int)blockDim.x);
}

// Orders each bucket by (view, pixel) so the gathers sum in a fixed order. With a view mask, the buckets that
// hold two entries of one view (the only ones filled out of order) sort themselves in global memory. Without
// one, a block takes 256 consecutive buckets, whose entries are contiguous: when they fit, the block stages them
// in shared memory with coalesced loads, each thread insertion-sorts its bucket there, and the block writes
// them back coalesced; a larger group sorts in global memory, one bucket per thread.
constexpr int kSortBuckets = 256, kSortCap = 8192;

__device__ __forceinline__ void insertion_sort(unsigned int *a, unsigned int s, unsigned int e) {
    for (unsigned int i = s + 1; i < e; ++i) {
        const unsigned int key = a[i];
        unsigned int j = i;
        while (j > s && a[j - 1] > key) {
            a[j] = a[j - 1];
            --j;
        }
        a[j] = key;
    }
}

__global__ void __launch_bounds__(kSortBuckets) k_bucket_sort(int nb, const unsigned int *__restrict__ start,
                                                              const unsigned long long *__restrict__ mask, int mw,
                                                              unsigned int *__restrict__ entries) {
    pdl_wait();
    __shared__ unsigned int buf[kSortCap];
    const int b0 = blockIdx.x * kSortBuckets, b1 = min(b0 + kSortBuckets, nb), b = b0 + (int)threadIdx.x;
    // with a view mask only the buckets with two entries of one view need the sort: each sorts itself in place
    if (mask) {
        if (b < b1 && bucket_dup(start, mask, mw, nb, b)) insertion_sort(entries, start[b], start[b + 1]);
        return;
    }
    const unsigned int S = start[b0], E = start[b1];
    if (E - S <= (unsigned int)kSortCap) {
        for (unsigned int i = threadIdx.x; i < E - S; i += kSortBuckets) buf[i] = entries[S + i];
        __syncthreads();
        if (b < b1) insertion_sort(buf, start[b] - S, start[b + 1] - S);
        __syncthreads();
        for (unsigned int i = threadIdx.x; i < E - S; i += kSortBuckets) entries[S + i] = buf[i];
    } else if (b < b1) {
        insertion_sort(entries, start[b], start[b + 1]);
    }
}

// Exclusive scan of unsigned counts: each block scans kScanPer * kScanBlock counts (kScanPer per thread: a
// thread's own prefix, then warp shuffles over the thread totals and one warp over the warp totals) and writes its
// total; k_scan_finish then adds to every block the totals of the blocks before it. Integer sums: the result does
// not depend on the order.
constexpr int kScanBlock = 1024, kScanPer = 4, kScanSpan = kScanBlock * kScanPer;

__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(int nb, const unsigned int *__restrict__ in,
                                                            unsigned int *__restrict__ out,
                                                            unsigned int *__restrict__ block_sums) {
    pdl_wait();
    pdl_trigger();
    __shared__ unsigned int warp_tot[kScanBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int i0 = blockIdx.x * kScanSpan + threadIdx.x * kScanPer;
    unsigned int v[kScanPer];
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) v[j] = (i0 + j < nb) ? in[i0 + j] : 0u;
    unsigned int t = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) t += v[j];
    unsigned int incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        unsigned int w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    unsigned int run = (wid > 0 ? warp_tot[wid - 1] : 0u) + incl - t;  // exclusive prefix of this thread
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        if (i0 + j < nb) out[i0 + j] = run;
        run += v[j];
    }
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = warp_tot[31];
}

// Adds to block b's exclusive scan the sum of the totals of blocks 0 .. b - 1; out[nb] = the grand total.
// zero (optional): the scanned counts, cleared here for their next use as cursors (k_scan_blocks has read them)
__global__ void __launch_bounds__(kScanBlock) k_scan_finish(int nb, unsigned int *__restrict__ out,
                                                            const unsigned int *__restrict__ block_sums,
                                                            unsigned int *__restrict__ zero) {
    pdl_wait();
    pdl_trigger();
    __shared__ unsigned int red[kScanBlock / 32];
    unsigned int s = 0;
    for (int j = threadIdx.x; j < (int)blockIdx.x; j += kScanBlock) s += block_sums[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned int t = (threadIdx.x < kScanBlock / 32) ? red[threadIdx.x] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    const unsigned int off = red[0];
    const int i0 = blockIdx.x * kScanSpan + threadIdx.x * kScanPer;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
        if (i0 + j < nb) {
            out[i0 + j] += off;
            if (zero) zero[i0 + j] = 0u;
        }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[nb] = off + block_sums[blockIdx.x];
}

// ====================================================================== per-source gathers (v = A u)
// Weighted residual e = w * (A_i U - v_i) over the gather set, and the intensity energy
// sum sigma^2 w (A_i U - v_i)^2 (vtv_sr_dataterm_intensities sources/optimization.cu:1871-1903 and
// coco_vtv_sr_primal_energy_unstructured :1560-1608). Outside the gather set A_i U = 0.
// splat_set: the residual over the splat set instead, zero elsewhere (the corrected IBR_color objective, whose
// gradient splats over the same set).
template <int KS>
__global__ void __launch_bounds__(256) k_residual(int V, int n, int W, int H, int dsf, const float *__restrict__ U,
                                                  const float *__restrict__ img, const float *__restrict__ tau,
                                                  const float *__restrict__ wgt, float s2,
                                                  float *__restrict__ res, double *__restrict__ partial,
                                                  int splat_set) {
    __shared__ double red[8];
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    const size_t N = (size_t)W * H;
    double e = 0.0;
    if (m < n) {
        const float tx = tau[(size_t)v * 2 * n + m], ty = tau[(size_t)v * 2 * n + n + m];
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        if (in_gather(tx, ty, W, H)) {
            Footprint fp;
            footprint<KS>(tx, ty, dsf, W, H, fp);
#pragma unroll
            for (int j = 0; j < KS; ++j)
#pragma unroll
                for (int i = 0; i < KS; ++i) {
                    const int x = fp.x0 + j, y = fp.y0 + i;
                    if (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1) {
                        const float A = fp.A[KS * i + j];
                        const size_t o = (size_t)y * W + x;
                        a0 += A * __ldg(U + o);
                        a1 += A * __ldg(U + N + o);
                        a2 += A * __ldg(U + 2 * N + o);
                    }
                }
        }
        const float *iv = img + (size_t)v * 3 * n;
        const float w = (splat_set && !in_splat(tx, ty, W, H)) ? 0.f : wgt[(size_t)v * n + m];
        const float d0 = a0 - iv[m], d1 = a1 - iv[n + m], d2 = a2 - iv[2 * n + m];
        float *rv = res + (size_t)v * 3 * n;
        rv[m] = d0 * w;
        rv[n + m] = d1 * w;
        rv[2 * n + m] = d2 * w;
        e = (double)s2 * (double)w * ((double)d0 * d0 + (double)d1 * d1 + (double)d2 * d2);
    }
    const double s = block_sum<256>(e, red);
    if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// Angular and deformation weights of every source pixel (coco_vtv_sr_compute_weights_unstructured,
// sources/optimization.cu:1094-1163; vtv_sr_angular_weights_device and vtv_sr_gold_deform_weights_device,
// vtv_sr_kernels_unstructured.cu:174-266): w = 1/(sg^2 + sigma^2) * deform with sg = clamp(A_i grad) . dpart.
// GATHER = false: the target gradient is identically zero (gx == nullptr), so the gather through A is skipped
// at compile time and the kernel keeps few registers.
template <int KS, typename TW, bool GATHER>
__global__ void __launch_bounds__(256, GATHER ? 1 : 8) k_weights(int V, int n, int w, int h, int W, int H, int dsf,
                                                 const float *__restrict__ gx, const float *__restrict__ gy,
                                                 const float *__restrict__ tau, const float *__restrict__ dp,
                                                 float sigma, float thr, TW *__restrict__ wgt) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    if (m >= n) return;
    const float *tx = tau + (size_t)v * 2 * n, *ty = tx + n;
    // every load the pixel can need, issued together (neighbour indices clamped to the view; the clamped values
    // are read only where the neighbour exists)
    int mx, my;
    pixel_of(m, w, n, __frcp_rn((float)w), mx, my);
    const int ml = mx > 0 ? m - 1 : m, mr = mx < w - 1 ? m + 1 : m;
    const int mu = my > 0 ? m - w : m, md = my < h - 1 ? m + w : m;
    const float txm = __ldg(tx + m), tym = __ldg(ty + m);
    const float txl = __ldg(tx + ml), tyl = __ldg(ty + ml), txr = __ldg(tx + mr), tyr = __ldg(ty + mr);
    const float txu = __ldg(tx + mu), tyu = __ldg(ty + mu), txd = __ldg(tx + md), tyd = __ldg(ty + md);
    // (no dp: dtau/dz taken as 0, for callers whose gathered gradient is 0 anyway)
    const float dpx = dp ? __ldg(dp + (size_t)v * 2 * n + m) : 0.f;
    const float dpy = dp ? __ldg(dp + (size_t)v * 2 * n + n + m) : 0.f;
    float ax = 0.f, ay = 0.f;
    if (GATHER && in_gather(txm, tym, W, H)) {
        Footprint fp;
        footprint<KS>(txm, tym, dsf, W, H, fp);
#pragma unroll
        for (int j = 0; j < KS; ++j)
#pragma unroll
            for (int i = 0; i < KS; ++i) {
                const int x = fp.x0 + j, y = fp.y0 + i;
                if (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1) {
                    const float A = fp.A[KS * i + j];
                    const size_t o = (size_t)y * W + x;
                    ax += A * __ldg(gx + o);
                    ay += A * __ldg(gy + o);
                }
            }
    }
    // angular weight
    const float norm = sqrtf(ax * ax + ay * ay);
    if (norm > thr) {
        ax = ax / norm * thr;
        ay = ay / norm * thr;
    }
    float sg = ax * dpx + ay * dpy;
    if (sg > 0.5f) sg = 0.5f;
    const float ang = 1.0f / (sg * sg + sigma * sigma);
    // deformation weight
    auto out = [&](float x, float y) { return x < 0.f || x > (float)W || y < 0.f || y > (float)H; };
    float def;
    if (out(txm, tym)) def = 0.0f;
    else if (mx == 0 || my == 0 || mx == w - 1 || my == h - 1) def = 1.0f;
    else if (out(txl, tyl) || out(txr, tyr) || out(txu, tyu) || out(txd, tyd)) def = 1.0f;
    else {
        const float Dxx = 0.5f * (txr - txl);
        const float Dyx = 0.5f * (tyr - tyl);
        const float Dxy = 0.5f * (txd - txu);
        const float Dyy = 0.5f * (tyd - tyu);
        const float N = fabsf(Dxx * Dyy - Dxy * Dyx);
        def = (N > 1.0f) ? 1.0f / N : 1.0f;
    }
    stv(wgt + (size_t)v * n + m, ang * def);
}

// ====================================================================== A^T gathers (per target pixel)
// (SplatSrc and splat_accumulate live in device_common.cuh)

// Coverage and visibility (coco_vtv_setup_visibility_mask sources/optimization.cu:33-135):
// cov = sum A, vis = cov >= 1.
template <int KS>
__global__ void k_coverage(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                           const unsigned int *__restrict__ entries, const float *__restrict__ tau,
                           float *__restrict__ cov, uint8_t *__restrict__ vis) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    SplatSrc src{{nullptr, nullptr, nullptr}, {0, 0, 0}, nullptr};
    float acc[3], norm;
    splat_accumulate<KS, 0>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    const size_t o = (size_t)y * W + x;
    cov[o] = norm;
    vis[o] = (norm < 1.0f) ? 0 : 1;
}

// Visibility of IBR_gradient (setup_target_visibility, sources/gradientIBR.cu:40-83): some splatted tap
// with a non-zero raw overlap.
template <int KS>
__global__ void k_vis_any(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                          const unsigned int *__restrict__ entries, const float *__restrict__ tau,
                          uint8_t *__restrict__ vis) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    bool any = false;
#pragma unroll
    for (int i = 0; i < KS; ++i)
#pragma unroll
        for (int j = 0; j < KS; ++j) {
            const int ax = x - j, ay = y - i;
            const size_t b = (size_t)(ay + KS - 1) * BW + (ax + KS - 1);
            const unsigned int s = start[b], e = start[b + 1];
            for (unsigned int k = s; k < e && !any; ++k) {
                const unsigned int ent = entries[k];
                const int v = (int)(ent >> 24), m = (int)(ent & 0xFFFFFFu);
                const float tx = tau[(size_t)v * 2 * n + m], ty = tau[(size_t)v * 2 * n + n + m];
                if (footprint_raw<KS>(tx, ty, dsf, j, i, ax, ay) != 0.0f) any = true;
            }
        }
    vis[(size_t)y * W + x] = any ? 1 : 0;
}

// IBR_gradient set-up in one traversal of the inverse map (per target pixel):
//   visibility   setup_target_visibility (sources/gradientIBR.cu:40-83): some splatted raw overlap != 0;
//   weighted average of compute_initial_image (:724-808): U = sum w A v / sum w A;
//   gradient splat of init_u_gradient (:833-920): (gx, gy, mask) = sum A (Sobel_x, Sobel_y, w) / sum A,
//   mask scaled by sigma^2.
// img: per view [3][n]; vgrad: per view [2][n] (Sobel of the view luminance); wgt: per view [n].
struct SetupAcc {
    float u0 = 0.f, u1 = 0.f, u2 = 0.f, wn = 0.f;  // weighted average
    float g0 = 0.f, g1 = 0.f, g2 = 0.f, nrm = 0.f;  // gradient splat
    bool any = false;
    __device__ __forceinline__ void add(float A, float raw, float w, float c0, float c1, float c2, float s0, float s1) {
        any |= (raw != 0.0f);
        const float wA = w * A;
        wn += wA;
        u0 += wA * c0;
        u1 += wA * c1;
        u2 += wA * c2;
        nrm += A;
        g0 += A * s0;
        g1 += A * s1;
        g2 += A * w;
    }
    __device__ __forceinline__ void store(size_t o, size_t N, float s2, uint8_t *vis, float *U, float *gx, float *gy,
                                          float *mask) {
        vis[o] = any ? 1 : 0;
        if (wn != 0.f) {
            u0 /= wn;
            u1 /= wn;
            u2 /= wn;
        }
        U[o] = u0;
        U[N + o] = u1;
        U[2 * N + o] = u2;
        if (nrm != 0.f) {
            g0 /= nrm;
            g1 /= nrm;
            g2 /= nrm;
        }
        gx[o] = g0;
        gy[o] = g1;
        mask[o] = g2 * s2;
    }
};

// The set-up of one target pixel reading every entry straight from global memory.
template <int KS, typename TS>
__device__ __forceinline__ void gradient_setup_global(int x, int y, int W, int H, int n, int dsf, int BW,
                                                      const unsigned int *__restrict__ start,
                                                      const unsigned int *__restrict__ entries,
                                                      const float *__restrict__ tau, const TS *__restrict__ img,
                                                      const TS *__restrict__ vgrad, const TS *__restrict__ wgt,
                                                      SetupAcc &acc) {
#pragma unroll
    for (int i = 0; i < KS; ++i) {
#pragma unroll
        for (int j = 0; j < KS; ++j) {
            const int ax = x - j, ay = y - i;
            const size_t b = (size_t)(ay + KS - 1) * BW + (ax + KS - 1);
            const unsigned int s = __ldg(start + b), e = __ldg(start + b + 1);
            for (unsigned int k = s; k < e; ++k) {
                const unsigned int ent = __ldg(entries + k);
                const int v = (int)(ent >> 24), m = (int)(ent & 0xFFFFFFu);
                const float tx = __ldg(tau + (size_t)v * 2 * n + m), ty = __ldg(tau + (size_t)v * 2 * n + n + m);
                float raw;
                const float A = footprint_tap<KS>(tx, ty, dsf, W, H, ax, ay, j, i, raw);
                const TS *iv = img + (size_t)v * 3 * n;
                const TS *gv = vgrad + (size_t)v * 2 * n;
                acc.add(A, raw, ldv(wgt + (size_t)v * n + m), ldv(iv + m), ldv(iv + n + m), ldv(iv + 2 * n + m),
                        ldv(gv + m), ldv(gv + n + m));
            }
        }
    }
}

// Anchor-row form (KS <= 3). The entries of one anchor bucket reach a KS x KS block of target pixels, so
// instead of every target pixel re-reading the entries of its KS^2 buckets, a lane reads each entry of its
// buckets once and accumulates all KS^2 taps in registers (partials P[i][j][field]).
// A warp owns 64 consecutive anchors of one anchor row, starting at an even column: lane l takes anchor 2l in
// pass 0 and anchor 2l + 1 in pass 1, and owns pixel columns 2l and 2l + 1. With dsf 2 most source pixels of a
// box-decimated view land on even anchors, so one pass per parity makes a warp wait for its longest even bucket
// plus its longest odd bucket, not twice the longest of both. Pixel x of tap row i sums tap j of anchor x - j:
//   column 2l:      (P0[0] of 2l + P0[2] of 2l - 2) + P1[1] of 2l - 1
//   column 2l + 1:   P0[1] of 2l + (P1[0] of 2l + 1 + P1[2] of 2l - 1)
// (P0 / P1: the pass-0 / pass-1 partials; the left terms come from lane l - 1 by shuffle). The block then adds
// the KS tap rows of each pixel from shared memory. Every sum has a fixed order, so results are deterministic.
// Lane 0's columns lack their left anchors, so a warp outputs 62 pixels. The footprint norm is the product of
// the row and column overlap sums (the KS^2 taps are an outer product), and a tap is visible when both of its
// overlaps are non-zero. Fields: 0 w A, 1-3 w A v, 4 A, 5-6 A Sobel, 7 visibility. The mask sum (A w) is
// field 0: the same products added in the same order.
constexpr int kGrWarps = 8;
constexpr int kGrTXO = 62;  // output pixels per warp row
constexpr int kGrNF = 8;    // fields per tap-row partial

template <int KS>
constexpr size_t gradient_rows_smem() {
    return sizeof(float) * (kGrWarps * 2 - (KS - 1)) * KS * kGrNF * kGrTXO;
}

template <int KS, typename TS>
__global__ void __launch_bounds__(kGrWarps * 32, 2) k_gradient_setup_rows(int W, int H, int n, int dsf, int BW,
                                                                       const unsigned int *__restrict__ start,
                                                                       const unsigned int *__restrict__ entries,
                                                                       const float *__restrict__ tau,
                                                                       const TS *__restrict__ img,
                                                                       const TS *__restrict__ vgrad,
                                                                       const TS *__restrict__ wgt, float s2,
                                                                       uint8_t *__restrict__ vis,
                                                                       float *__restrict__ U, float *__restrict__ gx,
                                                                       float *__restrict__ gy,
                                                                       float *__restrict__ mask) {
    constexpr int TY = kGrWarps * 2 - (KS - 1);  // output pixel rows per block
    constexpr int NA = 7;                        // accumulated fields
    extern __shared__ float gr_part[];           // [TY][KS][kGrNF][kGrTXO]: (pixel row, tap row, field, pixel)
    pdl_trigger();                               // the hole list, launched next, waits for this grid's completion
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * kGrTXO, y0 = blockIdx.y * TY;
    const int BH = H + KS - 1;
    const int lx = 2 * lane - 2;  // this lane's first pixel column inside the tile
    // warp w takes anchor rows 2w and 2w + 1: one of each parity (with dsf = 2 the populated anchors mostly sit
    // on even rows, so rows w and w + 8 would leave half the warps idle)
    for (int q = 0; q < 2; ++q) {
        const int rr = 2 * warp + q;
        const int ay = y0 - (KS - 1) + rr, by = ay + KS - 1;
        bool iny[KS];
#pragma unroll
        for (int i = 0; i < KS; ++i) iny[i] = (0 <= ay + i && ay + i <= H - 1);
#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            const int ax = x0 - 2 + 2 * lane + pass, bx = ax + KS - 1;
            bool inx[KS];
#pragma unroll
            for (int j = 0; j < KS; ++j) inx[j] = (0 <= ax + j && ax + j <= W - 1);
            float P[KS][KS][NA];
#pragma unroll
            for (int i = 0; i < KS; ++i)
#pragma unroll
                for (int j = 0; j < KS; ++j)
#pragma unroll
                    for (int f = 0; f < NA; ++f) P[i][j][f] = 0.f;
            unsigned int anyb = 0;
            if (bx >= 0 && bx < BW && by < BH) {
                const size_t b = (size_t)by * BW + bx;
                const unsigned int s = __ldg(start + b), e = __ldg(start + b + 1);
                // software pipeline: the entry index three ahead and the source data of the next two entries
                // are in flight while the current entry is accumulated
                struct Src {
                    float tx, ty, w, c0, c1, c2, s0, s1;
                };
                auto fetch = [&](unsigned int ent) {
                    const int v = (int)(ent >> 24), m = (int)(ent & 0xFFFFFFu);
                    const TS *iv = img + (size_t)v * 3 * n;
                    const TS *gv = vgrad + (size_t)v * 2 * n;
                    Src d;
                    d.tx = __ldg(tau + (size_t)v * 2 * n + m);
                    d.ty = __ldg(tau + (size_t)v * 2 * n + n + m);
                    d.w = ldv(wgt + (size_t)v * n + m);
                    d.c0 = ldv(iv + m);
                    d.c1 = ldv(iv + n + m);
                    d.c2 = ldv(iv + 2 * n + m);
                    d.s0 = ldv(gv + m);
                    d.s1 = ldv(gv + n + m);
                    return d;
                };
                Src cur = {}, nx1 = {};
                unsigned int ent_next = 0;
                if (s < e) cur = fetch(__ldg(entries + s));
                if (s + 1 < e) nx1 = fetch(__ldg(entries + s + 1));
                if (s + 2 < e) ent_next = __ldg(entries + s + 2);
                for (unsigned int k = s; k < e; ++k) {
                    Src nx2 = {};
                    if (k + 2 < e) nx2 = fetch(ent_next);
                    if (k + 3 < e) ent_next = __ldg(entries + k + 3);
                    const float w = cur.w, c0 = cur.c0, c1 = cur.c1, c2 = cur.c2, s0 = cur.s0, s1 = cur.s1;
                    const float px = cur.tx - 0.5f, py = cur.ty - 0.5f;
                    cur = nx1;
                    nx1 = nx2;
                    float dx[KS], dy[KS], sx = 0.f, sy = 0.f;
                    unsigned int xb = 0;
#pragma unroll
                    for (int t = 0; t < KS; ++t) {
                        dx[t] = inx[t] ? fp_overlap(t, KS, ax + t, px, dsf) : 0.0f;
                        dy[t] = iny[t] ? fp_overlap(t, KS, ay + t, py, dsf) : 0.0f;
                        sx = __fadd_rn(sx, dx[t]);
                        sy = __fadd_rn(sy, dy[t]);
                        xb |= (dx[t] != 0.0f) ? 1u << t : 0u;
                    }
                    // one reciprocal per entry; A = (dx * (1 / norm)) * dy is within a few ulps of dx dy / norm
                    const float norm = __fmul_rn(sx, sy);
                    const float inv = (norm != 0.0f) ? __frcp_rn(norm) : 1.0f;
                    const float w0 = w * c0, w1 = w * c1, w2 = w * c2;
#pragma unroll
                    for (int i = 0; i < KS; ++i) {
                        anyb |= (dy[i] != 0.0f) ? xb << (i * KS) : 0u;
                        const float yi = __fmul_rn(dy[i], inv);
#pragma unroll
                        for (int j = 0; j < KS; ++j) {
                            const float A = __fmul_rn(dx[j], yi);
                            P[i][j][0] += w * A;
                            P[i][j][1] += A * w0;
                            P[i][j][2] += A * w1;
                            P[i][j][3] += A * w2;
                            P[i][j][4] += A;
                            P[i][j][5] += A * s0;
                            P[i][j][6] += A * s1;
                        }
                    }
                }
            }
            // tap rows of this pass into shared memory: pass 0 stores, pass 1 adds (same lane, same slots)
#pragma unroll
            for (int i = 0; i < KS; ++i) {
                const int py = ay + i - y0;  // output pixel row inside the tile
                float c0[NA], c1[NA];
                unsigned int v0, v1;
                const unsigned int bi = anyb >> (i * KS);
                const unsigned int bl = __shfl_up_sync(0xffffffffu, bi, 1);
                if (pass == 0) {
#pragma unroll
                    for (int f = 0; f < NA; ++f) {
                        const float left = (KS == 3) ? __shfl_up_sync(0xffffffffu, P[i][KS - 1][f], 1) : 0.0f;
                        c0[f] = (KS == 3) ? P[i][0][f] + left : P[i][0][f];
                        c1[f] = P[i][1][f];
                    }
                    v0 = (bi & 1u) | ((KS == 3) ? (bl >> 2) & 1u : 0u);
                    v1 = (bi >> 1) & 1u;
                } else {
#pragma unroll
                    for (int f = 0; f < NA; ++f) {
                        c0[f] = __shfl_up_sync(0xffffffffu, P[i][1][f], 1);
                        const float left = (KS == 3) ? __shfl_up_sync(0xffffffffu, P[i][KS - 1][f], 1) : 0.0f;
                        c1[f] = (KS == 3) ? P[i][0][f] + left : P[i][0][f];
                    }
                    v0 = (bl >> 1) & 1u;
                    v1 = (bi & 1u) | ((KS == 3) ? (bl >> 2) & 1u : 0u);
                }
                if (lane >= 1 && py >= 0 && py < TY) {
                    float *row = gr_part + (size_t)(py * KS + i) * kGrNF * kGrTXO + lx;
#pragma unroll
                    for (int f = 0; f < NA; ++f) {
                        float2 *d = reinterpret_cast<float2 *>(row + f * kGrTXO);
                        if (pass == 0) {
                            *d = make_float2(c0[f], c1[f]);
                        } else {
                            const float2 o = *d;
                            *d = make_float2(o.x + c0[f], o.y + c1[f]);
                        }
                    }
                    float2 *dv = reinterpret_cast<float2 *>(row + NA * kGrTXO);
                    if (pass == 0) {
                        *dv = make_float2(v0 ? 1.f : 0.f, v1 ? 1.f : 0.f);
                    } else {
                        const float2 o = *dv;
                        *dv = make_float2((o.x != 0.f || v0) ? 1.f : 0.f, (o.y != 0.f || v1) ? 1.f : 0.f);
                    }
                }
            }
        }
    }
    __syncthreads();
    // add the tap rows of every pixel in order and normalise (as SetupAcc::store)
    const size_t N = (size_t)W * H;
    for (int p = threadIdx.x; p < TY * kGrTXO; p += kGrWarps * 32) {
        const int px = p % kGrTXO, ly = p / kGrTXO, x = x0 + px, y = y0 + ly;
        if (x >= W || y >= H) continue;
        SetupAcc acc;
        float any = 0.f;
#pragma unroll
        for (int i = 0; i < KS; ++i) {
            const float *c = gr_part + (size_t)(ly * KS + i) * kGrNF * kGrTXO + px;
            acc.wn += c[0 * kGrTXO];
            acc.u0 += c[1 * kGrTXO];
            acc.u1 += c[2 * kGrTXO];
            acc.u2 += c[3 * kGrTXO];
            acc.nrm += c[4 * kGrTXO];
            acc.g0 += c[5 * kGrTXO];
            acc.g1 += c[6 * kGrTXO];
            any += c[7 * kGrTXO];
        }
        acc.g2 = acc.wn;
        acc.any = any != 0.f;
        acc.store((size_t)y * W + x, N, s2, vis, U, gx, gy, mask);
    }
}

// Per-pixel form for KS > 3 (too many register partials for the anchor-row form).
template <int KS, typename TS>
__global__ void __launch_bounds__(256) k_gradient_setup_px(int W, int H, int n, int dsf, int BW,
                                                           const unsigned int *__restrict__ start,
                                                           const unsigned int *__restrict__ entries,
                                                           const float *__restrict__ tau, const TS *__restrict__ img,
                                                           const TS *__restrict__ vgrad,
                                                           const TS *__restrict__ wgt, float s2,
                                                           uint8_t *__restrict__ vis, float *__restrict__ U,
                                                           float *__restrict__ gx, float *__restrict__ gy,
                                                           float *__restrict__ mask) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    SetupAcc acc;
    gradient_setup_global<KS, TS>(x, y, W, H, n, dsf, BW, start, entries, tau, img, vgrad, wgt, acc);
    acc.store((size_t)y * W + x, (size_t)W * H, s2, vis, U, gx, gy, mask);
}

// Weighted average (coco_vtv_sr_compute_initial_image sources/optimization.cu:1300-1344):
// U = sum w A v / sum w A where the weight sum is non-zero.
template <int KS>
__global__ void k_initial_image(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                                const unsigned int *__restrict__ entries, const float *__restrict__ tau,
                                SplatSrc src, float *__restrict__ U, float *__restrict__ norm_out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    float acc[3], norm;
    splat_accumulate<KS, 3>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    const size_t o = (size_t)y * W + x, N = (size_t)W * H;
#pragma unroll
    for (int c = 0; c < 3; ++c) U[c * N + o] = (norm != 0.f) ? acc[c] / norm : acc[c];
    if (norm_out) norm_out[o] = norm;
}

// Input of the learned warm start, NHWC BF16 with kLearnChannels (48) channels per target pixel:
// [0..2] the anchor u0 (hole-filled weighted average), [3] gx, [4] gy (the splatted luminance gradient, one plane
// each; zero in the last column / row, which the normal equations never read, and clamped to [-1, 1], the range
// of finite differences of [0, 1] images), [5] visibility, [6 + 3 v .. 8 + 3 v] view v splatted alone
// (sum A w v / sum A w over its own footprints), [30 + v] view v's share of the total splat weight, for the first
// kLearnViews views; [38..40] the CG's initial residual at u0 per channel, r0 = grad^T g + Delta u0 (FP32, the
// operator's boundary rules, clamped to [-4, 4]); [41..47] zero. Per-view accumulators live in shared memory (one
// column per thread), so the view index of an entry needs no register indexing.
// Each entry's tap is computed alone, not through footprint_tap's KS^2 products: the footprint is an outer product,
// so its norm is the product of the in-image row and column overlap sums, and the tap (j, i) is
// dx_j * (dy_i / norm) with one reciprocal (within a few ulps of footprint_tap's quotient, as in the set-up's
// anchor-row form). The gather is a chain of dependent loads (bucket bounds, entry, the view's data), so all KS x KS
// buckets' bounds and first entries are loaded up front (a row's KS buckets are contiguous) and each bucket's loop
// keeps the entry two ahead and the next entry's data in flight.
template <int KS, typename TS>
__global__ void __launch_bounds__(256, 4) k_learn_input(int W, int H, int n, int dsf, int BW,
                                                     const unsigned int *__restrict__ start,
                                                     const unsigned int *__restrict__ entries,
                                                     const float *__restrict__ tau, const TS *__restrict__ img,
                                                     const TS *__restrict__ wgt, const float *__restrict__ U,
                                                     const float *__restrict__ gx, const float *__restrict__ gy,
                                                     const uint8_t *__restrict__ vis, __nv_bfloat16 *__restrict__ out) {
    __shared__ float acc[kLearnViews * 4][256];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    // a block covers 64 x 4 pixels; warp w takes the columns of parity w & 1 of row w >> 1, so that the lanes of a
    // warp scan buckets of one anchor parity (with dsf 2 most entries sit on even anchors)
    const int x = blockIdx.x * 64 + 2 * threadIdx.x + (threadIdx.y & 1), y = blockIdx.y * 4 + (threadIdx.y >> 1);
#pragma unroll
    for (int i = 0; i < kLearnViews * 4; ++i) acc[i][t] = 0.f;
    if (x >= W || y >= H) return;
    // row i's anchors x - KS + 1 .. x are buckets r .. r + KS - 1 of that row: column j's bucket is r + KS - 1 - j
    unsigned int bs[KS][KS + 1];
#pragma unroll
    for (int i = 0; i < KS; ++i) {
        const size_t r = (size_t)(y - i + KS - 1) * BW + x;
#pragma unroll
        for (int q = 0; q <= KS; ++q) bs[i][q] = __ldg(start + r + q);
    }
    constexpr unsigned int kNone = 0xFFFFFFFFu;  // view 255: past the first views
    auto ok = [](unsigned int ent) { return (int)(ent >> 24) < kLearnViews; };
    // every bucket's first entry, loaded together
    unsigned int first[KS][KS];
#pragma unroll
    for (int i = 0; i < KS; ++i)
#pragma unroll
        for (int j = 0; j < KS; ++j)
            first[i][j] = bs[i][KS - 1 - j] < bs[i][KS - j] ? __ldg(entries + bs[i][KS - 1 - j]) : kNone;
    struct Src {
        float px, py, w, c0, c1, c2;
    };
    auto fetch = [&](unsigned int ent) {
        const size_t v = ent >> 24, m = ent & 0xFFFFFFu;
        Src d;
        d.px = __ldg(tau + v * 2 * n + m) - 0.5f;
        d.py = __ldg(tau + v * 2 * n + n + m) - 0.5f;
        d.w = ldv(wgt + v * n + m);
        d.c0 = ldv(img + (v * 3 + 0) * n + m);
        d.c1 = ldv(img + (v * 3 + 1) * n + m);
        d.c2 = ldv(img + (v * 3 + 2) * n + m);
        return d;
    };
#pragma unroll
    for (int i = 0; i < KS; ++i) {
        const int ay = y - i;
        bool iny[KS];
#pragma unroll
        for (int q = 0; q < KS; ++q) iny[q] = (0 <= ay + q && ay + q <= H - 1);
#pragma unroll
        for (int j = 0; j < KS; ++j) {
            const int ax = x - j;
            bool inx[KS];
#pragma unroll
            for (int q = 0; q < KS; ++q) inx[q] = (0 <= ax + q && ax + q <= W - 1);
            // software pipeline: the entry two ahead and the view data of the next entry are in flight while the
            // current entry is added
            const unsigned int s0 = bs[i][KS - 1 - j], e0 = bs[i][KS - j];
            unsigned int cur = first[i][j];
            if (!ok(cur)) continue;
            unsigned int nxt = s0 + 1 < e0 ? __ldg(entries + s0 + 1) : kNone;
            Src d = fetch(cur);
            for (unsigned int k = s0;; ++k) {
                const unsigned int n2 = (ok(nxt) && k + 2 < e0) ? __ldg(entries + k + 2) : kNone;
                Src dn = {};
                if (ok(nxt)) dn = fetch(nxt);
                const int v = (int)(cur >> 24);
                float sx = 0.f, sy = 0.f, dxj = 0.f, dyi = 0.f;
#pragma unroll
                for (int q = 0; q < KS; ++q) {
                    const float dx = inx[q] ? fp_overlap(q, KS, ax + q, d.px, dsf) : 0.f;
                    const float dy = iny[q] ? fp_overlap(q, KS, ay + q, d.py, dsf) : 0.f;
                    sx = __fadd_rn(sx, dx);
                    sy = __fadd_rn(sy, dy);
                    if (q == j) dxj = dx;
                    if (q == i) dyi = dy;
                }
                const float norm = __fmul_rn(sx, sy);
                const float inv = (norm != 0.0f) ? __frcp_rn(norm) : 1.0f;
                const float A = __fmul_rn(dxj, __fmul_rn(dyi, inv)) * d.w;
                acc[v * 4 + 3][t] += A;
                acc[v * 4 + 0][t] += A * d.c0;
                acc[v * 4 + 1][t] += A * d.c1;
                acc[v * 4 + 2][t] += A * d.c2;
                if (!ok(nxt)) break;  // entries ascend by view: the rest of the bucket are later views
                cur = nxt;
                nxt = n2;
                d = dn;
            }
        }
    }
    const size_t o = (size_t)y * W + x, N = (size_t)W * H;
    float f[kLearnChannels];
#pragma unroll
    for (int c = 0; c < kLearnChannels; ++c) f[c] = 0.f;
    const float gxo = gx[o], gyo = gy[o];
    const float gxl = x > 0 ? gx[o - 1] : 0.f, gyu = y > 0 ? gy[o - W] : 0.f;
    f[3] = x < W - 1 ? fminf(fmaxf(gxo, -1.f), 1.f) : 0.f;
    f[4] = y < H - 1 ? fminf(fmaxf(gyo, -1.f), 1.f) : 0.f;
    f[5] = vis[o] ? 1.f : 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float *u = U + c * N;
        const float uc = u[o];
        float lx, ly;
        if (x == 0) lx = uc - u[o + 1] + gxo;
        else if (x < W - 1) lx = 2.f * uc - u[o - 1] - u[o + 1] + gxo - gxl;
        else lx = uc - u[o - 1] - gxl;
        if (y == 0) ly = uc - u[o + W] + gyo;
        else if (y < H - 1) ly = 2.f * uc - u[o - W] - u[o + W] + gyo - gyu;
        else ly = uc - u[o - W] - gyu;
        f[c] = uc;
        f[38 + c] = fminf(fmaxf(-(lx + ly), -4.f), 4.f);
    }
    // quotients as products with one reciprocal each (within an ulp or two of the division; stored as BF16); a
    // divisor below 1e-30, whose reciprocal could overflow, divides
    auto quot = [](float num, float den, float rden) {
        return den >= 1e-30f ? num * rden : (den > 0.f ? num / den : 0.f);
    };
    float total = 0.f;
#pragma unroll
    for (int v = 0; v < kLearnViews; ++v) total += acc[v * 4 + 3][t];
    const float rtotal = total >= 1e-30f ? __frcp_rn(total) : 0.f;
#pragma unroll
    for (int v = 0; v < kLearnViews; ++v) {
        const float a = acc[v * 4 + 3][t];
        const float ra = a >= 1e-30f ? __frcp_rn(a) : 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) f[6 + 3 * v + c] = quot(acc[v * 4 + c][t], a, ra);
        f[6 + 3 * kLearnViews + v] = quot(a, total, rtotal);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(out + o * kLearnChannels);
#pragma unroll
    for (int q = 0; q < kLearnChannels / 8; ++q) {
        uint4 u;
        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
        for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[8 * q + 2 * i], f[8 * q + 2 * i + 1]);
        dst[q] = u;
    }
}

// Data-term gradient and the proximal data F (vtv_sr_dataterm_intensities :1953-1963 and
// vtv_sr_ista_step_unstructured :1785-1812): G = alpha sigma^2 sum A e / sum A, F = clamp(U + fs clamp(G)).
// With a gradient term (gt.resg set, vtv_sr_dataterm_gradients sources/optimization.cu:1969-2116) the
// residuals of the gradients are splatted too (same entries, same coverage) and
// G += beta * (-step) * [sigma^2 if gw_type] * sum A resg / sum A.
template <int KS>
__global__ void k_dataterm_F(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                             const unsigned int *__restrict__ entries, const float *__restrict__ tau, SplatSrc src,
                             float s2, float alpha, float fscale, const float *__restrict__ U,
                             float *__restrict__ F, float *__restrict__ G_out, GradTerm gt) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    float acc[3], norm;
    splat_accumulate<KS, 3>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    float accg[3] = {0.f, 0.f, 0.f}, normg = 0.f;
    if (gt.resg) {
        const size_t s3 = (size_t)3 * n;
        const SplatSrc sg{{gt.resg, gt.resg + n, gt.resg + 2 * (size_t)n}, {s3, s3, s3}, nullptr};
        splat_accumulate<KS, 3>(x, y, W, H, n, dsf, BW, start, entries, tau, sg, accg, normg);
    }
    const size_t o = (size_t)y * W + x, N = (size_t)W * H;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float gi = (norm != 0.f) ? acc[c] / norm : acc[c];
        gi *= s2;
        float G = 0.f + alpha * gi;
        if (gt.resg) {
            float gg = (normg != 0.f) ? accg[c] / normg : accg[c];
            if (gt.gw) gg *= s2;
            gg *= -gt.step;
            G += gt.beta * gg;
        }
        if (G_out) G_out[c * N + o] = G;
        G = fminf(1.0f, fmaxf(-1.0f, G));
        G *= fscale;
        G += U[c * N + o];
        F[c * N + o] = fminf(1.0f, fmaxf(0.0f, G));
    }
}

// Regulariser weight before the blur (coco_vtv_sr_init_regularizer_weight_unstructured
// sources/optimization.cu:2262-2319, vtv_sr_init_regularizer_weight_device vtv_sr_kernels.cu:1172-1195).
// norm_prior is the coverage accumulator's content before the call (never cleared upstream).
template <int KS>
__global__ void k_regweight(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                            const unsigned int *__restrict__ entries, const float *__restrict__ tau, SplatSrc src,
                            const float *__restrict__ norm_prior, float s2, float lmax, float lmin, float mmax,
                            float *__restrict__ g0, float *__restrict__ norm_out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    float acc[3], norm;
    splat_accumulate<KS, 1>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    const size_t o = (size_t)y * W + x;
    const float nm = (norm_prior ? norm_prior[o] : 0.f) + norm;
    float m = (nm != 0.f) ? acc[0] / nm : acc[0];
    m *= s2;
    g0[o] = (m == 0.0f) ? lmax : fmaxf(lmin, lmax - m / mmax);
    if (norm_out) norm_out[o] = nm;
}

// Gradient splatting of IBR_gradient (init_u_gradient sources/gradientIBR.cu:856-916): payload
// (Sobel_x, Sobel_y, weight) of every source pixel, normalised by the coverage; mask scaled by sigma^2.
template <int KS>
__global__ void k_u_gradient(int W, int H, int n, int dsf, int BW, const unsigned int *__restrict__ start,
                             const unsigned int *__restrict__ entries, const float *__restrict__ tau, SplatSrc src,
                             float s2, float *__restrict__ gx, float *__restrict__ gy, float *__restrict__ mask) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    float acc[3], norm;
    splat_accumulate<KS, 3>(x, y, W, H, n, dsf, BW, start, entries, tau, src, acc, norm);
    const size_t o = (size_t)y * W + x;
    if (norm != 0.f) {
        acc[0] /= norm;
        acc[1] /= norm;
        acc[2] /= norm;
    }
    gx[o] = acc[0];
    gy[o] = acc[1];
    mask[o] = acc[2] * s2;
}

// ====================================================================== stencils on the target
// Sobel of the luminance (vtv_sr_compute_gradient_device, vtv_sr_kernels_unstructured.cu:96-148); with a
// mask, interior pixels without a fully visible 3x3 neighbourhood keep the old content of gx/gy.
// Also used on source views (sources/gradientIBR_kernels.cuh:57-100, no mask); views are addressed with a
// per-blockIdx.z plane stride.
__global__ void k_sobel(int W, int H, const float *__restrict__ rgb, size_t in_stride, size_t ch_stride,
                        float *__restrict__ gx, float *__restrict__ gy, size_t out_stride,
                        const uint8_t *__restrict__ vis, double *__restrict__ abs_partial) {
    __shared__ double red[8];
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const float *r = rgb + (size_t)z * in_stride, *g = r + ch_stride, *b = g + ch_stride;
    float *ox = gx + (size_t)z * out_stride, *oy = gy + (size_t)z * out_stride;
    double a = 0.0;
    if (x < W && y < H) {
        const size_t o = (size_t)y * W + x;
        float gX = 0.f, gY = 0.f;
        bool write = true;
        if (0 < x && x < W - 1 && 0 < y && y < H - 1) {
            if (vis) {
                for (int dy = -1; dy <= 1 && write; ++dy)
                    for (int dx = -1; dx <= 1; ++dx)
                        if (!vis[o + (ptrdiff_t)dy * W + dx]) {
                            write = false;
                            break;
                        }
            }
            if (write) {
                // The reference evaluates the luminance as a double expression rounded to float; the
                // masked (target) Sobel does the same because the angular weights amplify its rounding.
                auto L = [&](int dx, int dy) {
                    const size_t q = o + (ptrdiff_t)dy * W + dx;
                    if (!vis) return lum(r[q], g[q], b[q]);
                    return (float)__dadd_rn(__dadd_rn(__dmul_rn(0.2126, (double)r[q]), __dmul_rn(0.7152, (double)g[q])),
                                            __dmul_rn(0.0722, (double)b[q]));
                };
                const float Ypp = L(-1, -1), Ypc = L(0, -1), Ypn = L(1, -1);
                const float Ycp = L(-1, 0), Ycn = L(1, 0);
                const float Ynp = L(-1, 1), Ync = L(0, 1), Ynn = L(1, 1);
                gX = (Ypn + 2.f * Ycn + Ynn - Ypp - 2.f * Ycp - Ynp) / 8.f;
                gY = (Ynp + 2.f * Ync + Ynn - Ypp - 2.f * Ypc - Ypn) / 8.f;
            }
        }
        if (write) {
            ox[o] = gX;
            oy[o] = gY;
        }
        if (abs_partial) a = fabs((double)ox[o]) + fabs((double)oy[o]);
    }
    if (abs_partial) {
        // block of 32x8 threads
        const int tid = threadIdx.y * blockDim.x + threadIdx.x;
        double v = a;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if ((tid & 31) == 0) red[tid >> 5] = v;
        __syncthreads();
        if (tid == 0) {
            double s = 0;
            for (int i = 0; i < (int)(blockDim.x * blockDim.y) / 32; ++i) s += red[i];
            abs_partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
        }
    }
}

// Reprojection of the 6 dual components onto the Frobenius ball of radius r (vtv_rof.cu:280-320).
__device__ __forceinline__ void rof_project(float p[6], float r) {
    float nn = 0.f;
    nn += p[0] * p[0] + p[2] * p[2] + p[4] * p[4];
    nn += p[1] * p[1] + p[3] * p[3] + p[5] * p[5];
    nn = sqrtf(nn);
    if (nn > r) {
        const float s = r / nn;
#pragma unroll
        for (int k = 0; k < 6; ++k) p[k] *= s;
    }
}

// All niter inner ROF iterations in one cooperative launch, temporally blocked. One iteration is the dual step
// p += sigma grad_fwd(U) (vtv_rof.cu:118-147), the reprojection of the 6 duals onto the ball of radius g
// (vtv_rof.cu:280-320) and the primal prox U = (tau F + lambda (U + tau div_bwd p)) / (tau + lambda)
// (cuda_kernels.cu:504-532). Each super-step runs up to kRofK iterations on a (kRofTX + 2 kRofK) x
// (kRofTY + 2 kRofK) region around a kRofTX x kRofTY tile and writes back the tile, whose values depend only on the
// region (the halo absorbs one pixel of staleness per iteration from each side). Super-steps read one global
// (U, P) pair and write the other, with a bounded grid barrier between them.
// Every thread owns the same PPT region pixels in every iteration (their coordinates and border flags are worked
// out once per tile): their U, P, F and g stay in registers, and shared memory carries only what the neighbours
// read, U (right and lower neighbours, in the dual step) and the x and y duals (left and upper neighbours, in the
// prox). The block sizes divide the region into equal shares, so no warp waits at the block barriers for a
// second pass of the others. K (iterations per super-step) and the block size are template parameters; the
// host picks an instantiation per image size with a timing autotuner (rof_autotune).
constexpr int kRofTX = 32, kRofTY = 16;
template <int K>
constexpr size_t rof_smem() {
    return (size_t)9 * (kRofTX + 2 * K) * (kRofTY + 2 * K) * sizeof(float);  // U 3, x duals 3, y duals 3
}

template <int kRofK, int kRofThreads>
__global__ void __launch_bounds__(kRofThreads) k_rof_persistent(int W, int H, int niter, float tau, float sigma,
                                                                float lam, float *U0, float *P0, float *U1,
                                                                float *P1, const float *__restrict__ F,
                                                                const float *__restrict__ g, GridBarrier gb) {
    constexpr int RX = kRofTX + 2 * kRofK, RY = kRofTY + 2 * kRofK, RN = RX * RY;
    constexpr int PPT = (RN + kRofThreads - 1) / kRofThreads;  // region pixels per thread
    extern __shared__ float sm[];
    float *sU = sm, *sPx = sm + 3 * RN, *sPy = sm + 6 * RN;
    const int tiles_x = (W + kRofTX - 1) / kRofTX, ntiles = tiles_x * ((H + kRofTY - 1) / kRofTY);
    const size_t N = (size_t)W * H;
    const float denom = tau + lam;
    // flags of an owned pixel: inside the image, its forward differences exist (x, y), its left / upper
    // neighbour's dual enters the divergence (inside the image and the region), and it is a tile pixel
    constexpr unsigned kIn = 1, kFx = 2, kFy = 4, kBx = 8, kBy = 16, kTile = 32, kRx = 64, kRy = 128;
    constexpr int kDistShift = 8;
    unsigned int gen = 0;
    int step = 0;
    for (int done = 0; done < niter; done += kRofK, ++step) {
        const int iters = min(kRofK, niter - done);
        const float *Ui = (step & 1) ? U1 : U0, *Pi = (step & 1) ? P1 : P0;
        float *Uo = (step & 1) ? U0 : U1, *Po = (step & 1) ? P0 : P1;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int rx0 = (t % tiles_x) * kRofTX - kRofK, ry0 = (t / tiles_x) * kRofTY - kRofK;
            float u[PPT][3], p[PPT][6], f[PPT][3], gg[PPT];
            unsigned int fl[PPT];
            size_t go[PPT];
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                const int i = threadIdx.x + k * kRofThreads;
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
                    if (lx >= kRofK && lx < kRofK + kRofTX && ly >= kRofK && ly < kRofK + kRofTY) f0 |= kTile;
                    // distance from the tile (Chebyshev, in pixels)
                    const int dx = max(max(kRofK - lx, lx - (kRofK + kRofTX - 1)), 0);
                    const int dy = max(max(kRofK - ly, ly - (kRofK + kRofTY - 1)), 0);
                    f0 |= (unsigned int)max(dx, dy) << kDistShift;
                }
                fl[k] = f0;
                const size_t o = in ? (size_t)gy * W + gx : 0;
                go[k] = o;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    u[k][c] = in ? __ldcg(Ui + c * N + o) : 0.f;
                    f[k][c] = in ? __ldg(F + c * N + o) : 0.f;
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) p[k][c] = in ? __ldcg(Pi + c * N + o) : 0.f;
                gg[k] = in ? __ldg(g + o) : 0.f;
                if (i < RN) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        sU[c * RN + i] = u[k][c];
                        sPx[c * RN + i] = p[k][2 * c];
                        sPy[c * RN + i] = p[k][2 * c + 1];
                    }
                }
            }
            __syncthreads();
            for (int it = 0; it < iters; ++it) {
                // Only the pixels the tile still depends on are updated: after iteration it the tile needs U within
                // distance iters - it - 1 of it (the prox), and that prox reads the duals one pixel further out
                // (the dual step, whose right and lower neighbours' U were updated in the iteration before).
                // dual step + reprojection: the pixel's own U and p, its right and lower neighbours' U
                const unsigned int dual_reach = (unsigned int)(iters - it) << kDistShift;
                const unsigned int prox_reach = (unsigned int)(iters - it - 1) << kDistShift;
#pragma unroll
                for (int k = 0; k < PPT; ++k) {
                    if (!(fl[k] & kIn) || (fl[k] & ~0xFFu) > dual_reach) continue;
                    const int i = threadIdx.x + k * kRofThreads;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float *su = sU + c * RN;
                        const float uc = u[k][c];
                        const float ur = (fl[k] & kRx) ? su[i + 1] : 0.f, ud = (fl[k] & kRy) ? su[i + RX] : 0.f;
                        const float gxv = (fl[k] & kFx) ? ur - uc : 0.f;
                        const float gyv = (fl[k] & kFy) ? ud - uc : 0.f;
                        p[k][2 * c] = p[k][2 * c] + sigma * gxv;
                        p[k][2 * c + 1] = p[k][2 * c + 1] + sigma * gyv;
                    }
                    rof_project(p[k], gg[k]);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        sPx[c * RN + i] = p[k][2 * c];
                        sPy[c * RN + i] = p[k][2 * c + 1];
                    }
                }
                __syncthreads();
                // primal prox: the pixel's new duals and its left / upper neighbours'
#pragma unroll
                for (int k = 0; k < PPT; ++k) {
                    if (!(fl[k] & kIn) || (fl[k] & ~0xFFu) > prox_reach) continue;
                    const int i = threadIdx.x + k * kRofThreads;
                    const int lx = i % RX, ly = i / RX;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        float st = p[k][2 * c] + p[k][2 * c + 1];
                        if (fl[k] & kBx) st -= (lx > 0) ? sPx[c * RN + i - 1] : 0.f;
                        if (fl[k] & kBy) st -= (ly > 0) ? sPy[c * RN + i - RX] : 0.f;
                        const float unew = u[k][c] + tau * st;
                        u[k][c] = (tau * f[k][c] + lam * unew) / denom;
                        sU[c * RN + i] = u[k][c];
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                if ((fl[k] & (kIn | kTile)) != (kIn | kTile)) continue;
                const size_t o = go[k];
#pragma unroll
                for (int c = 0; c < 3; ++c) Uo[c * N + o] = u[k][c];
#pragma unroll
                for (int c = 0; c < 6; ++c) Po[c * N + o] = p[k][c];
            }
            __syncthreads();  // the next tile overwrites the staged region
        }
        if (!grid_sync(gb, gen)) return;
    }
}

// Count of pixels whose largest channel change reaches thr (sr_compare_images,
// sources/super-resolution.cpp:16-51).
__global__ void k_moving(size_t N, const float *__restrict__ A, const float *__restrict__ B, float thr,
                         double *__restrict__ partial) {
    __shared__ double red[8];
    const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double c = 0.0;
    if (o < N) {
        float mx = 0.f;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) mx = fmaxf(mx, fabsf(A[ch * N + o] - B[ch * N + o]));
        c = (mx < thr) ? 0.0 : 1.0;
    }
    const double s = block_sum<256>(c, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Separable 11-tap Gaussian with clamp-to-edge (convolutionRowGPU / convolutionColumnGPU,
// cocolib/cocolib/cuda/cuda_convolutions.cu:110-238; kernel from gsl_kernel_gauss_1xn(11, 2.0)).
__constant__ float c_gauss[11];

// Both passes stage their block's rows (columns) with the 5-pixel halo in shared memory, clamped to the image as
// the taps are, and sum the 11 taps there in the order of the reference's loop.
constexpr int kBlurBX = 32, kBlurBY = 8, kBlurR = 5;

__global__ void __launch_bounds__(kBlurBX * kBlurBY) k_blur_rows(int W, int H, const float *__restrict__ in,
                                                                 float *__restrict__ out) {
    __shared__ float t[kBlurBY][kBlurBX + 2 * kBlurR];
    const int x0 = blockIdx.x * kBlurBX, y = min((int)(blockIdx.y * kBlurBY + threadIdx.y), H - 1);
    for (int i = threadIdx.x; i < kBlurBX + 2 * kBlurR; i += kBlurBX)
        t[threadIdx.y][i] = __ldg(in + (size_t)y * W + min(max(x0 - kBlurR + i, 0), W - 1));
    __syncthreads();
    const int x = x0 + threadIdx.x, yo = blockIdx.y * kBlurBY + threadIdx.y;
    if (x >= W || yo >= H) return;
    float s = 0.f;
#pragma unroll
    for (int k = -kBlurR; k <= kBlurR; ++k) s += t[threadIdx.y][threadIdx.x + kBlurR + k] * c_gauss[5 - k];
    out[(size_t)yo * W + x] = s;
}

__global__ void __launch_bounds__(kBlurBX * kBlurBY) k_blur_cols(int W, int H, const float *__restrict__ in,
                                                                 float *__restrict__ out) {
    __shared__ float t[kBlurBY + 2 * kBlurR][kBlurBX];
    const int x = min((int)(blockIdx.x * kBlurBX + threadIdx.x), W - 1), y0 = blockIdx.y * kBlurBY;
    for (int i = threadIdx.y; i < kBlurBY + 2 * kBlurR; i += kBlurBY)
        t[i][threadIdx.x] = __ldg(in + (size_t)min(max(y0 - kBlurR + i, 0), H - 1) * W + x);
    __syncthreads();
    const int xo = blockIdx.x * kBlurBX + threadIdx.x, y = y0 + threadIdx.y;
    if (xo >= W || y >= H) return;
    float s = 0.f;
#pragma unroll
    for (int k = -kBlurR; k <= kBlurR; ++k) s += t[threadIdx.y + kBlurR + k][threadIdx.x] * c_gauss[5 - k];
    out[(size_t)y * W + xo] = s;
}

// Deterministic final reduction of FP64 partials (single block).
__global__ void k_reduce_final(int count, const double *__restrict__ partial, double *__restrict__ out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) s += partial[i];
    const double t = block_sum<1024>(s, red);
    if (threadIdx.x == 0) *out = t;
}

// One energy-trace entry: the host's float expression lambda e_tv + alpha e_int (+ beta e_grad), without
// contraction (the host code is compiled with -ffp-contract=off).
__global__ void k_trace_energy(const double *__restrict__ sums, float lambda, float alpha, float beta, int grad,
                               double *__restrict__ dst) {
    float e = __fadd_rn(__fmul_rn(lambda, (float)sums[0]), __fmul_rn(alpha, (float)sums[1]));
    if (grad) e = __fadd_rn(e, __fmul_rn(beta, (float)sums[3]));
    *dst = (double)e;
}

// Elementwise helpers.
__global__ void k_fill_u8(size_t n, uint8_t *p, uint8_t v) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void k_premultiply_dpart(int V, int n, const float *__restrict__ dpart3, int dpart_channels,
                                    float *__restrict__ dp) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    if (m >= n) return;
    const float *src = dpart3 + (size_t)v * dpart_channels * n;
    const float sz = src[m];
    dp[(size_t)v * 2 * n + m] = src[n + m] * sz;
    dp[(size_t)v * 2 * n + n + m] = src[2 * n + m] * sz;
}

__global__ void k_copy_tau(int V, int n, const float *__restrict__ tau_in, int tau_channels,
                           float *__restrict__ tau) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    if (m >= n) return;
    const float *src = tau_in + (size_t)v * tau_channels * n;
    tau[(size_t)v * 2 * n + m] = src[m];
    tau[(size_t)v * 2 * n + n + m] = src[n + m];
}

// ====================================================================== host launchers
static inline dim3 grid2(int W, int H, dim3 b) { return dim3((W + b.x - 1) / b.x, (H + b.y - 1) / b.y); }


void launch_bucket_build(const Geometry &G, const float *tau, Buckets &B, cudaStream_t st, LaunchCounter &lc,
                         bool counted) {
    ProfScope _ps(lc, "bucket_build", st);
    const int ks = G.dsf + 1;
    // one block per (view, chunk of 256 * kBucketPer source pixels), views varying fastest: the blocks in flight
    // cover one band of source rows in every view, so the buckets they count into and fill (whose entries
    // interleave the views) stay in one band of the target, in L2, until every view's entry of a sector is in
    const dim3 b1(256), gs((unsigned)((G.n + 256 * kBucketPer - 1) / (256 * kBucketPer)) * (unsigned)G.V);
    if (!counted) {  // else k_tau has counted while writing tau
        cudaMemsetAsync(B.count, 0, sizeof(unsigned int) * B.nb, st);
        if (B.mask) cudaMemsetAsync(B.mask, 0, sizeof(unsigned long long) * B.nb * B.mask_words, st);
        k_bucket_count<<<gs, b1, 0, st>>>(G.V, G.n, G.W, G.H, G.dsf, B.BW, tau, B.count, B.mask, B.nb);
        lc.add(1);
    }
    // exclusive scan of the counts: block-local scans, then every block adds the sum of the block totals before
    // it (integer sums, so the result does not depend on the order) and the last block writes the total
    const int nblk = (B.nb + kScanSpan - 1) / kScanSpan;
    // programmatic launches: each kernel's launch overlaps the tail of the one before it; k_scan_finish clears
    // the counts for their use as k_bucket_fill's cursors
    launch_pdl(k_scan_blocks, dim3(nblk), dim3(kScanBlock), 0, st, B.nb, B.count, B.start, B.block_sums);
    launch_pdl(k_scan_finish, dim3(nblk), dim3(kScanBlock), 0, st, B.nb, B.start, B.block_sums, B.count);
    lc.add(2);
    launch_pdl(k_bucket_fill, gs, b1, 0, st, G.V, G.n, G.W, G.H, G.dsf, B.BW, tau, B.start, B.count, B.mask,
               B.mask_words, B.nb, B.entries);
    launch_pdl(k_bucket_sort, dim3((B.nb + kSortBuckets - 1) / kSortBuckets), dim3(kSortBuckets), 0, st, B.nb,
               B.start, B.mask, B.mask_words, B.entries);
    lc.add(2);
    (void)ks;
}

void launch_residual(const Geometry &G, const float *U, const float *img, const float *tau, const float *wgt, float s2,
                     float *res, double *partial, cudaStream_t st, LaunchCounter &lc, bool splat_set) {
    ProfScope _ps(lc, "residual", st);
    const dim3 b(256), g((G.n + 255) / 256, G.V);
    LFRV_KS_DISPATCH(G.dsf + 1, k_residual, g, b, st, G.V, G.n, G.W, G.H, G.dsf, U, img, tau, wgt, s2, res, partial,
                     splat_set ? 1 : 0);
    lc.add(1);
}
int residual_partials(const Geometry &G) { return ((G.n + 255) / 256) * G.V; }

template <typename TW>
static void weights_typed(const Geometry &G, const float *gx, const float *gy, const float *tau, const float *dp,
                          float sigma, float thr, TW *wgt, cudaStream_t st) {
    const dim3 b(256), g((G.n + 255) / 256, G.V);
#define LFRV_WEIGHTS(KS_)                                                                                          \
    if (gx)                                                                                                        \
        k_weights<KS_, TW, true><<<g, b, 0, st>>>(G.V, G.n, G.w, G.h, G.W, G.H, G.dsf, gx, gy, tau, dp, sigma, thr, wgt); \
    else                                                                                                           \
        k_weights<KS_, TW, false><<<g, b, 0, st>>>(G.V, G.n, G.w, G.h, G.W, G.H, G.dsf, gx, gy, tau, dp, sigma, thr, wgt);
    switch (G.dsf + 1) {
        case 2: LFRV_WEIGHTS(2) break;
        case 3: LFRV_WEIGHTS(3) break;
        case 4: LFRV_WEIGHTS(4) break;
        case 5: LFRV_WEIGHTS(5) break;
        default: break;
    }
#undef LFRV_WEIGHTS
}

void launch_weights(const Geometry &G, const float *gx, const float *gy, const float *tau, const float *dp, float sigma,
                    float thr, void *wgt, cudaStream_t st, LaunchCounter &lc, bool bf16) {
    ProfScope _ps(lc, "weights", st);
    if (bf16) weights_typed(G, gx, gy, tau, dp, sigma, thr, static_cast<__nv_bfloat16 *>(wgt), st);
    else weights_typed(G, gx, gy, tau, dp, sigma, thr, static_cast<float *>(wgt), st);
    lc.add(1);
}

static const dim3 kTile(32, 8);

void launch_coverage(const Geometry &G, const Buckets &B, const float *tau, float *cov, uint8_t *vis, cudaStream_t st,
                     LaunchCounter &lc) {
    LFRV_KS_DISPATCH(G.dsf + 1, k_coverage, grid2(G.W, G.H, kTile), kTile, st, G.W, G.H, G.n, G.dsf, B.BW, B.start,
                     B.entries, tau, cov, vis);
    lc.add(1);
}

void launch_vis_any(const Geometry &G, const Buckets &B, const float *tau, uint8_t *vis, cudaStream_t st,
                    LaunchCounter &lc) {
    LFRV_KS_DISPATCH(G.dsf + 1, k_vis_any, grid2(G.W, G.H, kTile), kTile, st, G.W, G.H, G.n, G.dsf, B.BW, B.start,
                     B.entries, tau, vis);
    lc.add(1);
}

void launch_initial_image(const Geometry &G, const Buckets &B, const float *tau, const float *img, const float *wgt,
                          float *U, float *norm, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "initial_image", st);
    const size_t s3 = (size_t)3 * G.n;
    SplatSrc src{{img, img + G.n, img + 2 * (size_t)G.n}, {s3, s3, s3}, wgt};
    LFRV_KS_DISPATCH(G.dsf + 1, k_initial_image, grid2(G.W, G.H, kTile), kTile, st, G.W, G.H, G.n, G.dsf, B.BW,
                     B.start, B.entries, tau, src, U, norm);
    lc.add(1);
}

template <typename TS>
static void learn_input_typed(const Geometry &G, const Buckets &B, const float *tau, const TS *img, const TS *wgt,
                              const float *U, const float *gx, const float *gy, const uint8_t *vis,
                              __nv_bfloat16 *out, cudaStream_t st) {
    const dim3 g((G.W + 63) / 64, (G.H + 3) / 4);  // 64 x 4 pixels per block of kTile (32 x 8) threads
    switch (G.dsf + 1) {
        case 2: k_learn_input<2, TS><<<g, kTile, 0, st>>>(G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries, tau, img, wgt, U, gx, gy, vis, out); break;
        case 3: k_learn_input<3, TS><<<g, kTile, 0, st>>>(G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries, tau, img, wgt, U, gx, gy, vis, out); break;
        case 4: k_learn_input<4, TS><<<g, kTile, 0, st>>>(G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries, tau, img, wgt, U, gx, gy, vis, out); break;
        case 5: k_learn_input<5, TS><<<g, kTile, 0, st>>>(G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries, tau, img, wgt, U, gx, gy, vis, out); break;
        default: break;
    }
}

void launch_learn_input(const Geometry &G, const Buckets &B, const float *tau, const void *img, const void *wgt,
                        const float *U, const float *gx, const float *gy, const uint8_t *vis, void *out,
                        cudaStream_t st, LaunchCounter &lc, bool bf16) {
    ProfScope _ps(lc, "learn_input", st);
    __nv_bfloat16 *o = static_cast<__nv_bfloat16 *>(out);
    if (bf16)
        learn_input_typed(G, B, tau, static_cast<const __nv_bfloat16 *>(img), static_cast<const __nv_bfloat16 *>(wgt),
                          U, gx, gy, vis, o, st);
    else
        learn_input_typed(G, B, tau, static_cast<const float *>(img), static_cast<const float *>(wgt), U, gx, gy, vis,
                          o, st);
    lc.add(1);
}

void launch_dataterm_F(const Geometry &G, const Buckets &B, const float *tau, const float *res, float s2, float alpha,
                       float fscale, const float *U, float *F, float *G_out, const GradTerm &gt, cudaStream_t st,
                       LaunchCounter &lc) {
    ProfScope _ps(lc, "dataterm", st);
    const size_t s3 = (size_t)3 * G.n;
    SplatSrc src{{res, res + G.n, res + 2 * (size_t)G.n}, {s3, s3, s3}, nullptr};
    LFRV_KS_DISPATCH(G.dsf + 1, k_dataterm_F, grid2(G.W, G.H, kTile), kTile, st, G.W, G.H, G.n, G.dsf, B.BW, B.start,
                     B.entries, tau, src, s2, alpha, fscale, U, F, G_out, gt);
    lc.add(1);
}

// cuda_laplacian_device (cocolib/cocolib/vtv/vtv_sr_kernels_unstructured.cu:720-760) without a visibility mask,
// on `planes` planes of W x H: mean of the in-image 4-neighbours (left, up, right, down) minus the centre.
__device__ __forceinline__ float laplacian_at(const float *u, int W, int H, int x, int y) {
    const size_t o = (size_t)y * W + x;
    float v = 0.f, wt = 0.f;
    if (x > 0) { v += u[o - 1]; wt += 1.f; }
    if (y > 0) { v += u[o - W]; wt += 1.f; }
    if (x < W - 1) { v += u[o + 1]; wt += 1.f; }
    if (y < H - 1) { v += u[o + W]; wt += 1.f; }
    v /= wt;
    v -= u[o];
    return v;
}

__global__ void k_laplacian(int W, int H, int planes, const float *__restrict__ in, float *__restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t N = (size_t)W * H, o = (size_t)y * W + x;
    for (int c = 0; c < planes; ++c) out[c * N + o] = laplacian_at(in + c * N, W, H, x, y);
}

// Residual of the gradient data term for every source pixel (vtv_sr_dataterm_gradients, optimization.cu:
// 2010-2069): dsf^2 A_i lap(U) - lap(v_i), times omega_i when gw_type != 0. lapU is 3 x N (k_laplacian).
template <int KS>
__global__ void __launch_bounds__(256) k_residual_grad(int V, int w, int h, int W, int H, int dsf,
                                                       const float *__restrict__ lapU, const float *__restrict__ img,
                                                       const float *__restrict__ tau, const float *__restrict__ wgt,
                                                       int gw, float *__restrict__ resg) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    const int n = w * h;
    if (m >= n) return;
    const size_t N = (size_t)W * H;
    const float tx = tau[(size_t)v * 2 * n + m], ty = tau[(size_t)v * 2 * n + n + m];
    float a[3] = {0.f, 0.f, 0.f};
    if (in_gather(tx, ty, W, H)) {
        Footprint fp;
        footprint<KS>(tx, ty, dsf, W, H, fp);
#pragma unroll
        for (int j = 0; j < KS; ++j)
#pragma unroll
            for (int i = 0; i < KS; ++i) {
                const int x = fp.x0 + j, y = fp.y0 + i;
                if (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1) {
                    const float A = fp.A[KS * i + j];
                    const size_t o = (size_t)y * W + x;
#pragma unroll
                    for (int c = 0; c < 3; ++c) a[c] += A * __ldg(lapU + c * N + o);
                }
            }
    }
    const float dsf2 = (float)(dsf * dsf);
    int mx, my;
    pixel_of(m, w, n, __frcp_rn((float)w), mx, my);
    const float *iv = img + (size_t)v * 3 * n;
    float *rv = resg + (size_t)v * 3 * n;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float d = a[c] * dsf2;
        d -= laplacian_at(iv + (size_t)c * n, w, h, mx, my);
        if (gw) d *= wgt[(size_t)v * n + m];
        rv[(size_t)c * n + m] = d;
    }
}

// Gradient term of the reference energy (coco_vtv_sr_primal_energy_unstructured, optimization.cu:1610-1700):
// per source pixel (A_i Sobel_x lum U - Sobel_x lum v_i)^2 + (same for y), times omega_i sigma^2 when
// gw_type != 0. ugrad: 2 x N (Sobel of the luminance of U, no mask); vgrad: per view 2 x n.
template <int KS>
__global__ void __launch_bounds__(256) k_energy_grad(int V, int n, int W, int H, int dsf,
                                                     const float *__restrict__ ugrad, const float *__restrict__ vgrad,
                                                     const float *__restrict__ tau, const float *__restrict__ wgt,
                                                     float s2, int gw, double *__restrict__ partial) {
    __shared__ double red[8];
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    const size_t N = (size_t)W * H;
    double e = 0.0;
    if (m < n) {
        const float tx = tau[(size_t)v * 2 * n + m], ty = tau[(size_t)v * 2 * n + n + m];
        float ax = 0.f, ay = 0.f;
        if (in_gather(tx, ty, W, H)) {
            Footprint fp;
            footprint<KS>(tx, ty, dsf, W, H, fp);
#pragma unroll
            for (int j = 0; j < KS; ++j)
#pragma unroll
                for (int i = 0; i < KS; ++i) {
                    const int x = fp.x0 + j, y = fp.y0 + i;
                    if (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1) {
                        const float A = fp.A[KS * i + j];
                        const size_t o = (size_t)y * W + x;
                        ax += A * __ldg(ugrad + o);
                        ay += A * __ldg(ugrad + N + o);
                    }
                }
        }
        const float *vg = vgrad + (size_t)v * 2 * n;
        float a = ax - vg[m], b = ay - vg[n + m];
        a = a * a;
        b = b * b;
        if (gw) {
            const float w = wgt[(size_t)v * n + m];
            a *= w;
            b *= w;
            a *= s2;
            b *= s2;
        }
        e = (double)a + (double)b;
    }
    const double s = block_sum<256>(e, red);
    if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

int energy_grad_partials(const Geometry &G) { return ((G.n + 255) / 256) * G.V; }

void launch_laplacian(int W, int H, int planes, const float *in, float *out, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "laplacian", st);
    k_laplacian<<<grid2(W, H, kTile), kTile, 0, st>>>(W, H, planes, in, out);
    lc.add(1);
}

void launch_residual_grad(const Geometry &G, const float *lapU, const float *img, const float *tau, const float *wgt,
                          int gw, float *resg, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "residual_grad", st);
    const dim3 b(256), g((G.n + 255) / 256, G.V);
    LFRV_KS_DISPATCH(G.dsf + 1, k_residual_grad, g, b, st, G.V, G.w, G.h, G.W, G.H, G.dsf, lapU, img, tau, wgt, gw,
                     resg);
    lc.add(1);
}

void launch_energy_grad(const Geometry &G, const float *ugrad, const float *vgrad, const float *tau, const float *wgt,
                        float s2, int gw, double *partial, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "energy_grad", st);
    const dim3 b(256), g((G.n + 255) / 256, G.V);
    LFRV_KS_DISPATCH(G.dsf + 1, k_energy_grad, g, b, st, G.V, G.n, G.W, G.H, G.dsf, ugrad, vgrad, tau, wgt, s2, gw,
                     partial);
    lc.add(1);
}

void launch_regweight(const Geometry &G, const Buckets &B, const float *tau, const float *wgt, const float *norm_prior,
                      float s2, float lmax, float lmin, float mmax, float *g0, float *norm_out, cudaStream_t st,
                      LaunchCounter &lc) {
    SplatSrc src{{wgt, nullptr, nullptr}, {(size_t)G.n, 0, 0}, nullptr};
    LFRV_KS_DISPATCH(G.dsf + 1, k_regweight, grid2(G.W, G.H, kTile), kTile, st, G.W, G.H, G.n, G.dsf, B.BW, B.start,
                     B.entries, tau, src, norm_prior, s2, lmax, lmin, mmax, g0, norm_out);
    lc.add(1);
}

void launch_u_gradient(const Geometry &G, const Buckets &B, const float *tau, const float *vgrad, const float *wgt,
                       float s2, float *gx, float *gy, float *mask, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "u_gradient", st);
    // vgrad: per view [2][n] (Sobel x, Sobel y); weights [V][n]
    SplatSrc src{{vgrad, vgrad + G.n, wgt}, {(size_t)2 * G.n, (size_t)2 * G.n, (size_t)G.n}, nullptr};
    LFRV_KS_DISPATCH(G.dsf + 1, k_u_gradient, grid2(G.W, G.H, kTile), kTile, st, G.W, G.H, G.n, G.dsf, B.BW, B.start,
                     B.entries, tau, src, s2, gx, gy, mask);
    lc.add(1);
}

template <int KS, typename TS>
static void gradient_setup_ks(const Geometry &G, const Buckets &B, const float *tau, const TS *img,
                              const TS *vgrad, const TS *wgt, float s2, uint8_t *vis, float *U, float *gx,
                              float *gy, float *mask, cudaStream_t st) {
    if constexpr (KS <= 3) {
        constexpr int TY = kGrWarps * 2 - (KS - 1);
        constexpr size_t smem = gradient_rows_smem<KS>();
        static std::once_flag once;
        std::call_once(once, [] {
            cudaFuncSetAttribute(k_gradient_setup_rows<KS, TS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        });
        const dim3 g((G.W + kGrTXO - 1) / kGrTXO, (G.H + TY - 1) / TY);
        k_gradient_setup_rows<KS, TS><<<g, kGrWarps * 32, smem, st>>>(G.W, G.H, G.n, G.dsf, B.BW, B.start, B.entries,
                                                                    tau, img, vgrad, wgt, s2, vis, U, gx, gy, mask);
    } else {
        k_gradient_setup_px<KS, TS><<<grid2(G.W, G.H, kTile), kTile, 0, st>>>(G.W, G.H, G.n, G.dsf, B.BW, B.start,
                                                                            B.entries, tau, img, vgrad, wgt, s2, vis,
                                                                            U, gx, gy, mask);
    }
}

template <typename TS>
static void gradient_setup_typed(const Geometry &G, const Buckets &B, const float *tau, const TS *img, const TS *vgrad,
                                 const TS *wgt, float s2, uint8_t *vis, float *U, float *gx, float *gy, float *mask,
                                 cudaStream_t st) {
    switch (G.dsf + 1) {
        case 2: gradient_setup_ks<2, TS>(G, B, tau, img, vgrad, wgt, s2, vis, U, gx, gy, mask, st); break;
        case 3: gradient_setup_ks<3, TS>(G, B, tau, img, vgrad, wgt, s2, vis, U, gx, gy, mask, st); break;
        case 4: gradient_setup_ks<4, TS>(G, B, tau, img, vgrad, wgt, s2, vis, U, gx, gy, mask, st); break;
        case 5: gradient_setup_ks<5, TS>(G, B, tau, img, vgrad, wgt, s2, vis, U, gx, gy, mask, st); break;
        default: break;
    }
}

void launch_gradient_setup(const Geometry &G, const Buckets &B, const float *tau, const void *img, const void *vgrad,
                           const void *wgt, float s2, uint8_t *vis, float *U, float *gx, float *gy, float *mask,
                           cudaStream_t st, LaunchCounter &lc, bool bf16) {
    ProfScope _ps(lc, "gradient_setup", st);
    if (bf16)
        gradient_setup_typed(G, B, tau, static_cast<const __nv_bfloat16 *>(img),
                             static_cast<const __nv_bfloat16 *>(vgrad), static_cast<const __nv_bfloat16 *>(wgt), s2,
                             vis, U, gx, gy, mask, st);
    else
        gradient_setup_typed(G, B, tau, static_cast<const float *>(img), static_cast<const float *>(vgrad),
                             static_cast<const float *>(wgt), s2, vis, U, gx, gy, mask, st);
    lc.add(1);
}

// Luminance Sobel of the views (the view path of k_sobel: no mask, zero on the border), FP32 or BF16 in and out.
// The luminance of a 32 x 32 tile and its one-pixel halo is computed once into shared memory (1.13 loads per
// pixel and plane instead of 9); each thread of a 32 x 8 block then takes four rows. The arithmetic is k_sobel's,
// so the results are the same bit for bit.
constexpr int kSobelTY = 32;

template <typename T>
__global__ void __launch_bounds__(256) k_view_sobel(int W, int H, const T *__restrict__ rgb, size_t in_stride,
                                                    size_t ch_stride, T *__restrict__ gx, T *__restrict__ gy,
                                                    size_t out_stride) {
    __shared__ float Ls[kSobelTY + 2][35];
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * kSobelTY, z = blockIdx.z;
    const T *r = rgb + (size_t)z * in_stride, *g = r + ch_stride, *b = g + ch_stride;
    const int t = threadIdx.y * 32 + threadIdx.x;
    for (int k = t; k < (kSobelTY + 2) * 34; k += 256) {
        const int ly = k / 34, lx = k - ly * 34, xx = x0 - 1 + lx, yy = y0 - 1 + ly;
        float L = 0.f;
        if (xx >= 0 && xx < W && yy >= 0 && yy < H) {
            const size_t q = (size_t)yy * W + xx;
            L = lum(ldv(r + q), ldv(g + q), ldv(b + q));
        }
        Ls[ly][lx] = L;
    }
    __syncthreads();
    const int x = x0 + threadIdx.x;
    if (x >= W) return;
#pragma unroll
    for (int j = 0; j < kSobelTY / 8; ++j) {
        const int ry = threadIdx.y + 8 * j, y = y0 + ry;
        if (y >= H) break;
        const int tx = threadIdx.x + 1, ty = ry + 1;
        float gX = 0.f, gY = 0.f;
        if (0 < x && x < W - 1 && 0 < y && y < H - 1) {
            const float Ypp = Ls[ty - 1][tx - 1], Ypc = Ls[ty - 1][tx], Ypn = Ls[ty - 1][tx + 1];
            const float Ycp = Ls[ty][tx - 1], Ycn = Ls[ty][tx + 1];
            const float Ynp = Ls[ty + 1][tx - 1], Ync = Ls[ty + 1][tx], Ynn = Ls[ty + 1][tx + 1];
            gX = (Ypn + 2.f * Ycn + Ynn - Ypp - 2.f * Ycp - Ynp) / 8.f;
            gY = (Ynp + 2.f * Ync + Ynn - Ypp - 2.f * Ypc - Ypn) / 8.f;
        }
        const size_t o = (size_t)y * W + x;
        stv(gx + (size_t)z * out_stride + o, gX);
        stv(gy + (size_t)z * out_stride + o, gY);
    }
}

void launch_view_sobel_bf16(int W, int H, int count, const void *rgb, size_t in_stride, size_t ch_stride, void *gx,
                            void *gy, size_t out_stride, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "sobel", st);
    const dim3 b(32, 8), g((W + 31) / 32, (H + kSobelTY - 1) / kSobelTY, count);
    k_view_sobel<__nv_bfloat16><<<g, b, 0, st>>>(W, H, static_cast<const __nv_bfloat16 *>(rgb), in_stride, ch_stride,
                                                 static_cast<__nv_bfloat16 *>(gx), static_cast<__nv_bfloat16 *>(gy),
                                                 out_stride);
    lc.add(1);
}

void launch_sobel(int W, int H, int count, const float *rgb, size_t in_stride, size_t ch_stride, float *gx, float *gy,
                  size_t out_stride, const uint8_t *vis, double *abs_partial, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "sobel", st);
    const dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8, count);
    if (!vis && !abs_partial) {
        const dim3 gv((W + 31) / 32, (H + kSobelTY - 1) / kSobelTY, count);
        k_view_sobel<float><<<gv, b, 0, st>>>(W, H, rgb, in_stride, ch_stride, gx, gy, out_stride);
    } else {
        k_sobel<<<g, b, 0, st>>>(W, H, rgb, in_stride, ch_stride, gx, gy, out_stride, vis, abs_partial);
    }
    lc.add(1);
}
int sobel_partials(int W, int H) { return ((W + 31) / 32) * ((H + 7) / 8); }

// Instantiations the autotuner chooses from: (iterations per super-step, threads per block).
struct RofVariant {
    int K, threads;
    const void *kernel;
    size_t smem;
};
static const RofVariant kRofVariants[] = {
    // the region of K = 2, 4, 6, 8, 12 holds 720, 960, 1232, 1536, 2240 pixels: 2, 2, 2, 2 or 3, 4 per thread
    {2, 384, (const void *)k_rof_persistent<2, 384>, rof_smem<2>()},
    {4, 480, (const void *)k_rof_persistent<4, 480>, rof_smem<4>()},
    {6, 640, (const void *)k_rof_persistent<6, 640>, rof_smem<6>()},
    {8, 768, (const void *)k_rof_persistent<8, 768>, rof_smem<8>()},
    {8, 512, (const void *)k_rof_persistent<8, 512>, rof_smem<8>()},
    {12, 576, (const void *)k_rof_persistent<12, 576>, rof_smem<12>()},
};
int rof_variant_count() { return (int)(sizeof(kRofVariants) / sizeof(kRofVariants[0])); }
int rof_default_variant() { return 3; }  // K = 8, 768 threads

// Number of super-steps of variant v for niter iterations: the result is in (U1, P1) when it is odd.
int rof_persistent_steps(int niter, int v) { return (niter + kRofVariants[v].K - 1) / kRofVariants[v].K; }

cudaError_t launch_rof_persistent(int W, int H, int niter, float tau, float sigma, float lam, float *U0, float *P0,
                                  float *U1, float *P1, const float *F, const float *g, GridBarrier gb, int v,
                                  cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "rof_persistent", st);
    const RofVariant &R = kRofVariants[v];
    cudaError_t e = cudaFuncSetAttribute(R.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)R.smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, R.kernel, R.threads, R.smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int ntiles = ((W + kRofTX - 1) / kRofTX) * ((H + kRofTY - 1) / kRofTY);
    const int blocks = std::min(ntiles, sms * per_sm);
    void *args[] = {&W, &H, &niter, &tau, &sigma, &lam, &U0, &P0, &U1, &P1, (void *)&F, (void *)&g, &gb};
    lc.add(1);
    return cudaLaunchCooperativeKernel(R.kernel, dim3(blocks), dim3(R.threads), args, R.smem, st);
}

void launch_moving(size_t N, const float *A, const float *B, float thr, double *partial, cudaStream_t st,
                   LaunchCounter &lc) {
    k_moving<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, A, B, thr, partial);
    lc.add(1);
}
int moving_partials(size_t N) { return (int)((N + 255) / 256); }

void set_gaussian(const float k[11]) { cudaMemcpyToSymbol(c_gauss, k, sizeof(float) * 11); }

void launch_blur(int W, int H, const float *in, float *tmp, float *out, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "blur", st);
    const dim3 b(kBlurBX, kBlurBY);
    k_blur_rows<<<grid2(W, H, b), b, 0, st>>>(W, H, in, tmp);
    k_blur_cols<<<grid2(W, H, b), b, 0, st>>>(W, H, tmp, out);
    lc.add(2);
}

void launch_reduce_final(int count, const double *partial, double *out, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "reduce_final", st);
    k_reduce_final<<<1, 1024, 0, st>>>(count, partial, out);
    lc.add(1);
}

void launch_trace_energy(const double *sums, float lambda, float alpha, float beta, bool grad, double *dst,
                         cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "trace_energy", st);
    k_trace_energy<<<1, 1, 0, st>>>(sums, lambda, alpha, beta, grad ? 1 : 0, dst);
    lc.add(1);
}

void launch_premultiply_dpart(int V, int n, const float *dpart3, int ch, float *dp, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "premultiply_dpart", st);
    k_premultiply_dpart<<<dim3((n + 255) / 256, V), 256, 0, st>>>(V, n, dpart3, ch, dp);
    lc.add(1);
}

void launch_copy_tau(int V, int n, const float *tau_in, int ch, float *tau, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "copy_tau", st);
    k_copy_tau<<<dim3((n + 255) / 256, V), 256, 0, st>>>(V, n, tau_in, ch, tau);
    lc.add(1);
}

}  // namespace lfrv
