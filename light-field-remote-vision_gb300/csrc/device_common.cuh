// device_common.cuh -- device helpers shared by the lfrv kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace lfrv {

// Programmatic dependent launch. A kernel launched by launch_pdl may be scheduled while the kernel before it in
// the stream is finishing; pdl_wait() returns once that kernel has completed and its writes are visible, so a
// kernel calls it before touching anything earlier work wrote. pdl_trigger() lets the next such kernel be
// scheduled once every block of this one has issued it. Both are no-ops in a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... Params, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

constexpr int kMaxKs = 5;  // ks = dsf + 1, dsf <= 4

// ------------------------------------------------------------------ footprint of a source pixel
// Restates cuda_set_A_bilinear (cocolib/cocolib/vtv/vtv_sr_kernels_unstructured.cu:658-718): a dsf-wide
// box centred at tau - 0.5 covers ks x ks target pixels anchored at floor(px - dsf/2 + 1/2) with
// px = tau - 0.5; the weights are the box/pixel overlaps dx*dy, normalised by their sum over the
// in-image taps. The reference evaluates the anchor and the border overlaps in double and rounds each
// overlap once to float; the expressions below produce the same floats:
//   - px = tau - 0.5f is exact for 0.25 <= tau < 2^22 and otherwise rounded once, like the double path;
//   - for dsf = 1, 2 the anchor floor(px - (dsf-1)/2) is exact in float; other dsf use double;
//   - each overlap is a single rounding of the same exact value ((x + 1/2 + dsf/2) - px or
//     px - (x - 1/2 - dsf/2)).
// The products and the normalisation use round-to-nearest intrinsics so no FMA contraction changes them.
struct Footprint {
    int x0, y0;
    float A[kMaxKs * kMaxKs];  // entry ks*i + j: row offset i, column offset j
};

__device__ __forceinline__ int fp_anchor(float p, int dsf) {
    if (dsf == 1) return (int)floorf(p);
    if (dsf == 2) return (int)floorf(p - 0.5f);
    return (int)floor((double)p - 0.5 * dsf + 0.5);
}

__device__ __forceinline__ float fp_overlap(int k, int ks, int coord, float p, int dsf) {
    if (k == 0) return __fsub_rn((float)coord + 0.5f + 0.5f * (float)dsf, p);
    if (k == ks - 1) return __fsub_rn(p, (float)coord - 0.5f - 0.5f * (float)dsf);
    return 1.0f;
}

template <int KS>
__device__ __forceinline__ void footprint(float tx, float ty, int dsf, int W, int H, Footprint &fp) {
    const float px = tx - 0.5f, py = ty - 0.5f;
    fp.x0 = fp_anchor(px, dsf);
    fp.y0 = fp_anchor(py, dsf);
    float dxs[KS], dys[KS];
#pragma unroll
    for (int k = 0; k < KS; ++k) {
        dxs[k] = fp_overlap(k, KS, fp.x0 + k, px, dsf);
        dys[k] = fp_overlap(k, KS, fp.y0 + k, py, dsf);
    }
    float norm = 0.0f;
#pragma unroll
    for (int j = 0; j < KS; ++j) {
#pragma unroll
        for (int i = 0; i < KS; ++i) {
            const int x = fp.x0 + j, y = fp.y0 + i;
            const bool in = (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1);
            const float a = in ? __fmul_rn(dxs[j], dys[i]) : 0.0f;
            fp.A[KS * i + j] = a;
            norm = __fadd_rn(norm, a);
        }
    }
    if (norm != 0.0f) {
#pragma unroll
        for (int e = 0; e < KS * KS; ++e) fp.A[e] = __fdiv_rn(fp.A[e], norm);
    }
}

// Normalised weight of the single tap (j, i) of the footprint anchored at (x0, y0), with the float operations
// of footprint() (same products, same summation order of the norm, one division): the inverse-map gathers
// need one tap per visit. raw receives the un-normalised overlap dx*dy of that tap (0 when off-image).
// (J, I) are compile-time constants at every call site (fully unrolled loops), so the selection folds away.
template <int KS>
__device__ __forceinline__ float footprint_tap(float tx, float ty, int dsf, int W, int H, int x0, int y0, int J, int I,
                                               float &raw) {
    const float px = tx - 0.5f, py = ty - 0.5f;
    float dxs[KS], dys[KS];
#pragma unroll
    for (int k = 0; k < KS; ++k) {
        dxs[k] = fp_overlap(k, KS, x0 + k, px, dsf);
        dys[k] = fp_overlap(k, KS, y0 + k, py, dsf);
    }
    float norm = 0.0f, tap = 0.0f;
#pragma unroll
    for (int j = 0; j < KS; ++j) {
#pragma unroll
        for (int i = 0; i < KS; ++i) {
            const int x = x0 + j, y = y0 + i;
            const bool in = (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1);
            const float a = in ? __fmul_rn(dxs[j], dys[i]) : 0.0f;
            norm = __fadd_rn(norm, a);
            if (j == J && i == I) tap = a;
        }
    }
    raw = tap;
    return (norm != 0.0f) ? __fdiv_rn(tap, norm) : tap;
}

// The norm footprint_tap divides by, for the footprint anchored at (x0, y0): the same products summed in
// the same order (j outer, i inner), so footprint_tap_n(..., footprint_norm(...), raw) == footprint_tap(...).
template <int KS>
__device__ __forceinline__ float footprint_norm(float tx, float ty, int dsf, int W, int H, int x0, int y0) {
    const float px = tx - 0.5f, py = ty - 0.5f;
    float dxs[KS], dys[KS];
#pragma unroll
    for (int k = 0; k < KS; ++k) {
        dxs[k] = fp_overlap(k, KS, x0 + k, px, dsf);
        dys[k] = fp_overlap(k, KS, y0 + k, py, dsf);
    }
    float norm = 0.0f;
#pragma unroll
    for (int j = 0; j < KS; ++j) {
#pragma unroll
        for (int i = 0; i < KS; ++i) {
            const int x = x0 + j, y = y0 + i;
            const bool in = (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1);
            norm = __fadd_rn(norm, in ? __fmul_rn(dxs[j], dys[i]) : 0.0f);
        }
    }
    return norm;
}

// Tap (J, I) of the footprint anchored at (x0, y0) given its norm (from footprint_norm).
template <int KS>
__device__ __forceinline__ float footprint_tap_n(float tx, float ty, int dsf, int W, int H, int x0, int y0, int J,
                                                 int I, float norm, float &raw) {
    const float px = tx - 0.5f, py = ty - 0.5f;
    const int x = x0 + J, y = y0 + I;
    const bool in = (0 <= x && x <= W - 1 && 0 <= y && y <= H - 1);
    const float a = in ? __fmul_rn(fp_overlap(J, KS, x, px, dsf), fp_overlap(I, KS, y, py, dsf)) : 0.0f;
    raw = a;
    return (norm != 0.0f) ? __fdiv_rn(a, norm) : a;
}

// Raw overlap product of tap (j, i) (setup_visibility_mask, sources/gradientIBR_kernels.cuh:26-49).
template <int KS>
__device__ __forceinline__ float footprint_raw(float tx, float ty, int dsf, int j, int i, int x0, int y0) {
    const float px = tx - 0.5f, py = ty - 0.5f;
    return __fmul_rn(fp_overlap(j, KS, x0 + j, px, dsf), fp_overlap(i, KS, y0 + i, py, dsf));
}

// Gather set (cuda_convolution_nonsep_device_param, vtv_sr_kernels_unstructured.cu:286): tau in [0,W]x[0,H].
__device__ __forceinline__ bool in_gather(float tx, float ty, int W, int H) {
    return !(tx < 0.0f || ty < 0.0f || tx > (float)W || ty > (float)H);
}

// Splat set (vtv_sr_init_forward_warp_structure_unstructured, sources/optimization.cu:906-927):
// gather set and floor(tau - 0.5) inside the target.
__device__ __forceinline__ bool in_splat(float tx, float ty, int W, int H) {
    if (!in_gather(tx, ty, W, H)) return false;
    const int px = (int)floorf(tx - 0.5f), py = (int)floorf(ty - 0.5f);
    return !(px < 0 || py < 0 || px > W - 1 || py > H - 1);
}

// Column x and row y of pixel m of a w-wide view of n pixels, rw = RN(1/w). For n <= 2^21 the row is the float
// quotient (m + 1/2) rw truncated: its rounding error, below (m + 1/2) / w * 2^-23, is smaller than the distance
// 1/(2w) from (m + 1/2) / w to the nearest integer, so it equals the integer quotient, without the integer
// division's instruction sequence.
__device__ __forceinline__ void pixel_of(int m, int w, int n, float rw, int &x, int &y) {
    y = n <= (1 << 21) ? (int)(((float)m + 0.5f) * rw) : m / w;
    x = m - y * w;
}

// Inverse-map bucket of a source pixel with warp (tx, ty): its footprint anchor offset by ks - 1 on a grid of
// BW columns (-1: the pixel is not splatted).
__device__ __forceinline__ long long bucket_of(float tx, float ty, int W, int H, int dsf, int BW) {
    if (!in_splat(tx, ty, W, H)) return -1;
    const int ks = dsf + 1;
    const int x0 = fp_anchor(tx - 0.5f, dsf), y0 = fp_anchor(ty - 0.5f, dsf);
    return (long long)(y0 + ks - 1) * BW + (x0 + ks - 1);
}

// Luminance of the Sobel kernels (vtv_sr_kernels_unstructured.cu:121-130).
__device__ __forceinline__ float lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

// ------------------------------------------------------------------ block reductions (FP64)
// Deterministic: fixed shuffle tree inside a warp, fixed order across warps.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *smem /* >= NT/32 */) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NT / 32; ++i) s += smem[i];
    }
    __syncthreads();
    return s;  // valid in thread 0
}

// ------------------------------------------------------------------ bounded grid barrier
// For kernels launched cooperatively (all blocks co-resident). GridBarrier (kernels.h) holds a monotonically
// increasing arrival counter and an error flag, both zeroed before the launch. Every wait is bounded: after
// kSpinLimit polls (2^22 L2 round trips, a few seconds at most) the block sets *err and returns false;
// callers then exit, and the host reports LFRV_E_TIMEOUT.
constexpr long long kSpinLimit = 1ll << 22;

// nblocks: the blocks taking part (blocks 0 .. nblocks-1; the others must have returned before any barrier).
__device__ __forceinline__ bool grid_sync(const GridBarrier &gb, unsigned int &generation, unsigned int nblocks) {
    __syncthreads();
    generation += 1;
    bool ok = true;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        // release: the block's writes (ordered before this thread by the __syncthreads above) become visible to
        // every block that acquires the count after it; acquire: the other blocks' writes are visible here
        const unsigned int target = generation * nblocks;
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(gb.count) : "memory");
        // each poll is one L2 round trip; another block's error flag is read every 64th poll, so it does not
        // double the time between polls
        long long spins = 0;
        while (true) {
            unsigned int seen;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(seen) : "l"(gb.count) : "memory");
            if ((int)(seen - target) >= 0) break;
            if ((++spins & 63) == 0) {
                if (*((volatile int *)gb.err)) {
                    ok = false;
                    break;
                }
                if (spins > kSpinLimit) {
                    atomicExch(gb.err, 1);
                    ok = false;
                    break;
                }
            }
        }
    }
    __shared__ int s_ok;
    if (threadIdx.x == 0 && threadIdx.y == 0) s_ok = ok ? 1 : 0;
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ bool grid_sync(const GridBarrier &gb, unsigned int &generation) {
    return grid_sync(gb, generation, gridDim.x * gridDim.y);
}

// ---------------------------------------------------------------------- A^T gathers (per target pixel)
struct SplatSrc {
    const float *ch[3];   // payload channel c of view v at ch[c] + v * stride[c]
    size_t stride[3];
    const float *scale;   // optional per-source factor (weights), stride n per view
};

// Accumulates sum_entries A * payload and sum_entries A (times the optional scale) for target (x, y).
template <int KS, int NCH>
__device__ __forceinline__ void splat_accumulate(int x, int y, int W, int H, int n, int dsf, int BW,
                                                 const unsigned int *__restrict__ start,
                                                 const unsigned int *__restrict__ entries,
                                                 const float *__restrict__ tau, const SplatSrc &src, float acc[3],
                                                 float &norm) {
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] = 0.f;
    norm = 0.f;
#pragma unroll
    for (int i = 0; i < KS; ++i) {
#pragma unroll
        for (int j = 0; j < KS; ++j) {
            const int ax = x - j, ay = y - i;  // anchor whose tap (j, i) lands on (x, y)
            const size_t b = (size_t)(ay + KS - 1) * BW + (ax + KS - 1);
            const unsigned int s = __ldg(start + b), e = __ldg(start + b + 1);
            for (unsigned int k = s; k < e; ++k) {
                const unsigned int ent = __ldg(entries + k);
                const int v = (int)(ent >> 24), m = (int)(ent & 0xFFFFFFu);
                const float tx = __ldg(tau + (size_t)v * 2 * n + m), ty = __ldg(tau + (size_t)v * 2 * n + n + m);
                float raw;
                float A = footprint_tap<KS>(tx, ty, dsf, W, H, ax, ay, j, i, raw);
                if (src.scale) A = __ldg(src.scale + (size_t)v * n + m) * A;
                norm += A;
#pragma unroll
                for (int c = 0; c < NCH; ++c) acc[c] += A * __ldg(src.ch[c] + (size_t)v * src.stride[c] + m);
            }
        }
    }
}


// Instantiates a kernel template on the footprint size ks = dsf + 1 (2..5).
#define LFRV_KS_DISPATCH(ks, KERNEL, GRID, BLOCK, STREAM, ...)                          \
    switch (ks) {                                                                       \
        case 2: KERNEL<2><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;             \
        case 3: KERNEL<3><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;             \
        case 4: KERNEL<4><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;             \
        case 5: KERNEL<5><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;             \
        default: break;                                                                 \
    }

}  // namespace lfrv
