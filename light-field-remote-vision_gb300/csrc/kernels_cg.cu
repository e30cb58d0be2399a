// kernels_cg.cu -- IBR_gradient: hole filling and the Poisson conjugate gradient (sm_103a).
//
// hole_filling (sources/gradientIBR.cu:87-152, compute_laplacian sources/gradientIBR_kernels.cuh:553-590)
// runs Jacobi diffusion on the non-visible pixels only: the hole list is built once, every iteration reads
// the previous iterate and writes the holes of the other buffer (both buffers share the visible pixels).
//
// possion_conj_grad (sources/solver.cu:526-699) solves (lambda I - Delta_N) u = lambda u0 + grad^T g per
// channel. Its per-pixel operator (updateAlpha :201-310), initial residual (initConjGrad :361-505) and the
// updates (updateSolution :130-198, updateDir :508-523) are restated here; the dot products are FP64
// block partials reduced in a fixed order (the reference accumulates float atomics in arbitrary order).
#include <algorithm>
#include <cstring>
#include <mutex>

#include <cooperative_groups.h>
#include <cudaTypedefs.h>

#include "device_common.cuh"
#include "tma.cuh"
#include "kernels.h"
#include "lfrv_internal.h"

namespace lfrv {

namespace cg = cooperative_groups;

// Hole list in raster order: one warp per row counts its holes (ballot), one block scans the row counts,
// one warp per row writes its holes in order.
// Zero bytes of 16 visibility bytes (as a 16-bit mask, bit j = byte j) and their count.
__device__ __forceinline__ unsigned int zero_mask16(uint4 v) {
    const unsigned int w[4] = {v.x, v.y, v.z, v.w};
    unsigned int m = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const unsigned int e = __vcmpeq4(w[i], 0u);  // 0xff in every zero byte
#pragma unroll
        for (int j = 0; j < 4; ++j) m |= ((e >> (8 * j)) & 1u) << (4 * i + j);
    }
    return m;
}

__global__ void k_hole_rows(int W, int H, const uint8_t *__restrict__ vis, int *__restrict__ row_count) {
    pdl_wait();
    pdl_trigger();
    const int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (y >= H) return;
    int c = 0;
    if (W % 16 == 0) {
        // 16 pixels per lane and load (rows start on 16-byte boundaries)
        const uint8_t *row = vis + (size_t)y * W;
        for (int x = lane * 16; x < W; x += 512) c += __popc(zero_mask16(*reinterpret_cast<const uint4 *>(row + x)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    } else {
        for (int x0 = 0; x0 < W; x0 += 32) {
            const int x = x0 + lane;
            const bool hole = (x < W) && !vis[(size_t)y * W + x];
            c += __popc(__ballot_sync(0xffffffffu, hole));
        }
    }
    if (lane == 0) row_count[y] = c;
}

// Exclusive scan of H row counts in one block of 1024 threads (chunks of 1024 rows).
__global__ void k_hole_scan(int H, int *__restrict__ row_count, int *__restrict__ total) {
    pdl_wait();
    pdl_trigger();
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < H; base += 1024) {
        const int y = base + threadIdx.x;
        const int v = (y < H) ? row_count[y] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int wt = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, wt, o);
                if (lane >= o) wt += t;
            }
            warp_tot[lane] = wt;  // inclusive over warps
        }
        __syncthreads();
        const int before = (wid > 0) ? warp_tot[wid - 1] : 0;
        if (y < H) row_count[y] = carry + before + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_tot[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_hole_write(int W, int H, const uint8_t *__restrict__ vis, const int *__restrict__ row_start,
                             int *__restrict__ holes) {
    pdl_wait();
    const int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (y >= H) return;
    int k = row_start[y];
    if (W % 16 == 0) {
        // 16 pixels per lane and load; a lane's holes go after the holes of the lanes before it
        const uint8_t *row = vis + (size_t)y * W;
        for (int x0 = 0; x0 < W; x0 += 512) {
            const int x = x0 + lane * 16;
            const unsigned int m = (x < W) ? zero_mask16(*reinterpret_cast<const uint4 *>(row + x)) : 0u;
            const int c = __popc(m);
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            int at = k + incl - c;
            for (unsigned int r = m; r; r &= r - 1) holes[at++] = y * W + x + (__ffs(r) - 1);
            k += __shfl_sync(0xffffffffu, incl, 31);
        }
        return;
    }
    for (int x0 = 0; x0 < W; x0 += 32) {
        const int x = x0 + lane;
        const bool hole = (x < W) && !vis[(size_t)y * W + x];
        const unsigned int m = __ballot_sync(0xffffffffu, hole);
        if (hole) holes[k + __popc(m & ((1u << lane) - 1u))] = y * W + x;
        k += __popc(m);
    }
}

// One Jacobi step on the holes; partial = sum over holes of lap * U_new for channel 2 (the reference keeps
// the energy of the last channel).
__global__ void __launch_bounds__(256) k_hole_iter(int W, int H, const int *__restrict__ holes, int nholes,
                                                   const float *__restrict__ Uin, float *__restrict__ Uout,
                                                   double *__restrict__ partial) {
    __shared__ double red[8];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t N = (size_t)W * H;
    double e = 0.0;
    if (k < nholes) {
        const int o = holes[k];
        const int ox = o % W, oy = o / W;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float *u = Uin + c * N;
            float v = 0.f, wt = 0.f;
            if (ox > 0) { v += u[o - 1]; wt += 1.f; }
            if (oy > 0) { v += u[o - W]; wt += 1.f; }
            if (ox < W - 1) { v += u[o + 1]; wt += 1.f; }
            if (oy < H - 1) { v += u[o + W]; wt += 1.f; }
            v /= wt;
            const float lap = v - u[o];
            const float un = u[o] + lap;
            Uout[c * N + o] = un;
            if (c == 2) e = (double)(lap * un);
        }
    }
    const double s = block_sum<256>(e, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// ------------------------------------------------------------------ conjugate gradient
constexpr int kCgBX = 32, kCgBY = 8;

// Phase 0 of the corrected CG at pixel o: the initial residual r = b - A x with b = lambda u0 + grad^T g
// (initConjGrad, solver.cu:383-467) for the starting iterate x = U, and the energy
// F(x) = lambda/2 |x - u0|^2 + 1/2 |grad x - g|^2 there (the loop lowers it by each step's decrease, so the
// certified gap always refers to the current iterate). Without a separate anchor (U0 == nullptr) x = u0, as in
// the reference; with one, U holds a seed (the learned warm start) while u0 keeps the problem unchanged.
// acc[0..2] += r^2 per channel, acc[3] += the energy. cg_start_values returns the residual of pixel (x, y)
// (o = y W + x) per channel in rv3; cg_start_pixel stores it in r.
__device__ __forceinline__ void cg_start_values(int W, int H, size_t N, size_t o, int x, int y,
                                                const float *__restrict__ gX, const float *__restrict__ gY,
                                                const float *__restrict__ U, const float *__restrict__ U0,
                                                float lambda, float rv3[3], float acc[4]) {
    const float gxo = __ldg(gX + o), gyo = __ldg(gY + o);
    const float gxl = (x > 0) ? __ldg(gX + o - 1) : 0.f, gyu = (y > 0) ? __ldg(gY + o - W) : 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float *u = U + c * N;
        const float uc = __ldcg(u + o);
        float lx, ly;
        if (x == 0) lx = uc - __ldcg(u + o + 1) + gxo;
        else if (x < W - 1) lx = 2.f * uc - __ldcg(u + o - 1) - __ldcg(u + o + 1) + gxo - gxl;
        else lx = uc - __ldcg(u + o - 1) - gxl;
        if (y == 0) ly = uc - __ldcg(u + o + W) + gyo;
        else if (y < H - 1) ly = 2.f * uc - __ldcg(u + o - W) - __ldcg(u + o + W) + gyo - gyu;
        else ly = uc - __ldcg(u + o - W) - gyu;
        float rv = -(lx + ly);
        float e = 0.f;
        if (U0) {
            const float dv = __ldcg(U0 + c * N + o) - uc;
            rv += lambda * dv;
            e = lambda * dv * dv;
        }
        rv3[c] = rv;
        acc[c] += rv * rv;
        if (x < W - 1) {
            const float a = __ldcg(u + o + 1) - uc - gxo;
            e += a * a;
        }
        if (y < H - 1) {
            const float a = __ldcg(u + o + W) - uc - gyo;
            e += a * a;
        }
        acc[3] += 0.5f * e;
    }
}

__device__ __forceinline__ void cg_start_pixel(int W, int H, size_t N, size_t o, const float *__restrict__ gX,
                                               const float *__restrict__ gY, const float *__restrict__ U,
                                               const float *__restrict__ U0, float *__restrict__ r, float lambda,
                                               float acc[4]) {
    // 32-bit index arithmetic: images have fewer than 2^31 pixels
    const unsigned int ou = (unsigned int)o;
    const int y = (int)(ou / (unsigned int)W), x = (int)(ou - (unsigned int)y * (unsigned int)W);
    float rv[3];
    cg_start_values(W, H, N, o, x, y, gX, gY, U, U0, lambda, rv, acc);
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c * N + o] = rv[c];
}


__device__ __forceinline__ float cg_op(const float *d, int W, int H, int x, int y, size_t o, float lambda) {
    float lx, ly;
    if (x == 0) lx = d[o] - d[o + 1];
    else if (x < W - 1) lx = 2.f * d[o] - d[o - 1] - d[o + 1];
    else lx = d[o] - d[o - 1];
    if (y == 0) ly = d[o] - d[o + W];
    else if (y < H - 1) ly = 2.f * d[o] - d[o - W] - d[o + W];
    else ly = d[o] - d[o - W];
    return lambda * d[o] + lx + ly;
}

// partial layout: [3][nblocks]
__device__ __forceinline__ void cg_block3(double a0, double a1, double a2, double *partial) {
    __shared__ double red[3][8];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, off);
        a1 += __shfl_down_sync(0xffffffffu, a1, off);
        a2 += __shfl_down_sync(0xffffffffu, a2, off);
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = a0;
        red[1][tid >> 5] = a1;
        red[2][tid >> 5] = a2;
    }
    __syncthreads();
    if (tid == 0) {
        const int nb = gridDim.x * gridDim.y, b = blockIdx.y * gridDim.x + blockIdx.x;
        double s0 = 0, s1 = 0, s2 = 0;
        for (int i = 0; i < (kCgBX * kCgBY) / 32; ++i) {
            s0 += red[0][i];
            s1 += red[1][i];
            s2 += red[2][i];
        }
        partial[b] = s0;
        partial[nb + b] = s1;
        partial[2 * nb + b] = s2;
    }
}

// r0 = b - A x0 (initConjGrad, sources/solver.cu:383-467), d = r0, delta = r0 . r0; faithful counts the last
// row twice.
__global__ void __launch_bounds__(256) k_cg_init(int W, int H, const float *__restrict__ U, const float *__restrict__ gX,
                                                 const float *__restrict__ gY, float *__restrict__ r,
                                                 float *__restrict__ d, int faithful, double *__restrict__ partial) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const size_t N = (size_t)W * H;
    double acc[3] = {0, 0, 0};
    if (x < W && y < H) {
        const size_t o = (size_t)y * W + x;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float *u = U + c * N;
            float lx, ly;
            if (x == 0) lx = u[o] - u[o + 1] + gX[o];
            else if (x < W - 1) lx = 2.f * u[o] - u[o - 1] - u[o + 1] + gX[o] - gX[o - 1];
            else lx = u[o] - u[o - 1] - gX[o - 1];
            if (y == 0) ly = u[o] - u[o + W] + gY[o];
            else if (y < H - 1) ly = 2.f * u[o] - u[o - W] - u[o + W] + gY[o] - gY[o - W];
            else ly = u[o] - u[o - W] - gY[o - W];
            const float rv = -(lx + ly);
            r[c * N + o] = rv;
            d[c * N + o] = rv;
            acc[c] = (double)rv * rv * ((faithful && y == H - 1) ? 2.0 : 1.0);
        }
    }
    cg_block3(acc[0], acc[1], acc[2], partial);
}

// q = A d and d . q per channel.
__global__ void __launch_bounds__(256) k_cg_apply(int W, int H, const float *__restrict__ d, float lambda,
                                                  float *__restrict__ q, double *__restrict__ partial) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const size_t N = (size_t)W * H;
    double acc[3] = {0, 0, 0};
    if (x < W && y < H) {
        const size_t o = (size_t)y * W + x;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float qv = cg_op(d + c * N, W, H, x, y, o, lambda);
            q[c * N + o] = qv;
            acc[c] = (double)d[c * N + o] * qv;
        }
    }
    cg_block3(acc[0], acc[1], acc[2], partial);
}

// x += alpha d, r -= alpha q, r . r per channel (alpha per channel on the device).
__global__ void __launch_bounds__(256) k_cg_update(int W, int H, float3 alpha, const float *__restrict__ d, const float *__restrict__ q,
                                                   float *__restrict__ U, float *__restrict__ r,
                                                   double *__restrict__ partial) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const size_t N = (size_t)W * H;
    double acc[3] = {0, 0, 0};
    if (x < W && y < H) {
        const size_t o = (size_t)y * W + x;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float a = (c == 0) ? alpha.x : (c == 1) ? alpha.y : alpha.z;
            U[c * N + o] += a * d[c * N + o];
            const float rv = r[c * N + o] - a * q[c * N + o];
            r[c * N + o] = rv;
            acc[c] = (double)rv * rv;
        }
    }
    cg_block3(acc[0], acc[1], acc[2], partial);
}

__global__ void k_cg_dir(int W, int H, float3 beta, const float *__restrict__ r, float *__restrict__ d) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t N = (size_t)W * H, o = (size_t)y * W + x;
    d[o] = r[o] + beta.x * d[o];
    d[N + o] = r[N + o] + beta.y * d[N + o];
    d[2 * N + o] = r[2 * N + o] + beta.z * d[2 * N + o];
}

// Reduces nseg consecutive segments of `count` partials each (one block per segment).
__global__ void k_reduce_segments(int count, const double *__restrict__ partial, double *__restrict__ out) {
    __shared__ double red[32];
    const double *p = partial + (size_t)blockIdx.x * count;
    double s = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) s += p[i];
    const double t = block_sum<1024>(s, red);
    if (threadIdx.x == 0) out[blockIdx.x] = t;
}

// 1/2 ||u - u0||^2 + 1/2 ||grad u - g||^2 summed over channels (FP64), channel-summed partials in slot 0.
__global__ void __launch_bounds__(256) k_cg_energy(int W, int H, const float *__restrict__ U, const float *__restrict__ U0,
                                                   const float *__restrict__ gX, const float *__restrict__ gY,
                                                   double *__restrict__ partial) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const size_t N = (size_t)W * H;
    double acc[3] = {0, 0, 0};
    if (x < W && y < H) {
        const size_t o = (size_t)y * W + x;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float *u = U + c * N;
            const double dd = (double)u[o] - (double)U0[c * N + o];
            double e = 0.5 * dd * dd;
            if (x < W - 1) {
                const double a = (double)u[o + 1] - (double)u[o] - (double)gX[o];
                e += 0.5 * a * a;
            }
            if (y < H - 1) {
                const double a = (double)u[o + W] - (double)u[o] - (double)gY[o];
                e += 0.5 * a * a;
            }
            acc[c] = e;
        }
    }
    cg_block3(acc[0], acc[1], acc[2], partial);
}

// ====================================================================== persistent solvers
// One cooperative launch runs a whole iteration loop; phases are separated by the bounded grid barrier of
// device_common.cuh. Values written by other blocks inside the launch are read through L2 (__ldcg).
constexpr int kPersistThreads = 512;

// Sums of nslots slots of count FP64 values (slot s at p + s * stride) into out_smem[s], in FP64 and a fixed order:
// warp s takes slot s (lane l adds elements l, l + 32, ... in order, eight loads in flight at a time, then a
// shuffle tree). One warp per slot keeps each slot to one round trip to L2 and puts the slots' FP64 trees on
// separate warp schedulers (the FP64 pipe is narrow on this part). Needs a block of at least 32 * nslots threads.
__device__ void reduce_slots(const double *p, int count, size_t stride, int nslots, double *out_smem) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (wid < nslots) {
        const double *q = p + (size_t)wid * stride;
        double s = 0.0;
        for (int base = 0; base < count; base += 256) {
            double v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int i = base + lane + 32 * j;
                v[j] = i < count ? __ldcg(q + i) : 0.0;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) s += v[j];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) out_smem[wid] = s;
    }
    __syncthreads();
}

__device__ void block_reduce_partials(const double *partial, int count, int nslots, double *out_smem) {
    reduce_slots(partial, count, (size_t)count, nslots, out_smem);
}

// Block sum of up to 4 per-thread FP32 values into partial[slot * stride + blockIdx.x]: warp trees in FP32 (each
// lane holds a handful of terms, the slots interleaved), then warp s adds the warp sums of slot s in FP64 (a
// shuffle tree, fixed order). Every call site reaches a grid barrier next, whose leading block barrier orders
// these stores before the barrier's release and the shared buffer before its next use.
__device__ void block_partials_f(const float v[4], int nslots, double *partial, int stride) {
    __shared__ float red[4][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    float s[4] = {v[0], v[1], v[2], v[3]};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int sl = 0; sl < 4; ++sl) s[sl] += __shfl_down_sync(0xffffffffu, s[sl], o);
    if (lane == 0) {
#pragma unroll
        for (int sl = 0; sl < 4; ++sl) red[sl][wid] = s[sl];
    }
    __syncthreads();
    if (wid < nslots) {
        double t = lane < nw ? (double)red[wid][lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) partial[(size_t)wid * stride + blockIdx.x] = t;
    }
}

// Block sum of up to 4 per-thread values into partial[slot * stride + blockIdx.x] (stride: gridDim.x, or
// the number of participating blocks).
__device__ void block_partials(const double v[4], int nslots, double *partial, int stride) {
    __shared__ double red[kPersistThreads / 32][4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int sl = 0; sl < nslots; ++sl) {
        double s = v[sl];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[wid][sl] = s;
    }
    __syncthreads();
    if (threadIdx.x < nslots) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w][threadIdx.x];
        partial[(size_t)threadIdx.x * stride + blockIdx.x] = t;
    }
    __syncthreads();
}

__device__ __forceinline__ float ldcg_op(const float *d, int W, int H, int x, int y, size_t o, float lambda) {
    const float c = __ldcg(d + o);
    float lx, ly;
    if (x == 0) lx = c - __ldcg(d + o + 1);
    else if (x < W - 1) lx = 2.f * c - __ldcg(d + o - 1) - __ldcg(d + o + 1);
    else lx = c - __ldcg(d + o - 1);
    if (y == 0) ly = c - __ldcg(d + o + W);
    else if (y < H - 1) ly = 2.f * c - __ldcg(d + o - W) - __ldcg(d + o + W);
    else ly = c - __ldcg(d + o - W);
    return lambda * c + lx + ly;
}

// Tiles of the persistent CG: kTileX x kTileY pixels staged with a one-pixel halo.
constexpr int kTileX = 64, kTileY = 16, kHaloX = kTileX + 2, kHaloY = kTileY + 2;

// Operator of updateAlpha (sources/solver.cu:222-271) on a shared-memory tile: (tx, ty) is the pixel's tile
// position (halo included), (x, y) its image position for the one-sided border differences.
__device__ __forceinline__ float tile_op(const float (*t)[kHaloX], int tx, int ty, int x, int y, int W, int H,
                                         float lambda) {
    const float c = t[ty][tx];
    float lx, ly;
    if (x == 0) lx = c - t[ty][tx + 1];
    else if (x < W - 1) lx = 2.f * c - t[ty][tx - 1] - t[ty][tx + 1];
    else lx = c - t[ty][tx - 1];
    if (y == 0) ly = c - t[ty + 1][tx];
    else if (y < H - 1) ly = 2.f * c - t[ty - 1][tx] - t[ty + 1][tx];
    else ly = c - t[ty - 1][tx];
    return lambda * c + lx + ly;
}

// TMA form of the operator phases: each tile's halo arrives as one 3-D box per array (all 3 planes), x origin
// rounded down to a 16-byte boundary (x0 - 4), double-buffered so the next tile's box is in flight while the
// current one is used. Box rows are padded to a 128-byte multiple in shared memory.
constexpr int kBoxX = kTileX + 8, kBoxY = kTileY + 2, kBoxPlane = kBoxX * kBoxY;
constexpr unsigned kBoxBytes = 3u * kBoxPlane * sizeof(float);
constexpr unsigned kIntBytes = 3u * kTileX * kTileY * sizeof(float);  // interior box (no halo) of u or r
constexpr int kBoxStride = ((kBoxBytes + 127) / 128) * 128 / sizeof(float);  // floats between box buffers
constexpr size_t kCgTmaSmem = 6 * (size_t)kBoxStride * sizeof(float) + 128;   // 2 stages x 3 slots + alignment

// Operator of updateAlpha on a box in shared memory: f(i) is the value at box index i, ROW floats per box row.
template <int ROW = kBoxX, class F>
__device__ __forceinline__ float box_op(F f, int i, int x, int y, int W, int H, float lambda) {
    const float c = f(i);
    float lx, ly;
    if (x == 0) lx = c - f(i + 1);
    else if (x < W - 1) lx = 2.f * c - f(i - 1) - f(i + 1);
    else lx = c - f(i - 1);
    if (y == 0) ly = c - f(i + ROW);
    else if (y < H - 1) ly = 2.f * c - f(i - ROW) - f(i + ROW);
    else ly = c - f(i - ROW);
    return lambda * c + lx + ly;
}

// Thread 0 waits (bounded) for the stage's box; the block learns the outcome through shared memory, then every
// other thread observes the completed phase itself (it returns at once) so the box contents are visible to it.
__device__ __forceinline__ bool block_wait_box(uint64_t *bar, unsigned parity, int *s_flag) {
    if (threadIdx.x == 0) *s_flag = mbar_wait(bar, parity, kSpinLimit) ? 1 : 0;
    __syncthreads();
    const bool ok = *s_flag != 0;
    if (ok && threadIdx.x != 0) mbar_wait(bar, parity, kSpinLimit);
    return ok;
}

// Corrected CG of the IBR_gradient normal equations, all iterations in one launch. State layout (doubles):
// [0..2] delta, [3] E, [4] gap, [5] iterations, [6] status (0 ok, 1 barrier timeout).
// TMA = true reads the operator phases' tiles through the tensor maps of r, dA and dB (W a multiple of 4).
template <bool TMA>
__global__ void __launch_bounds__(kPersistThreads) k_cg_persistent(int W, int H, const float *__restrict__ gX,
                                                                   const float *__restrict__ gY, float *U,
                                                                   const float *U0, float *r,
                                                                   float *dA, float *dB, double *partA,
                                                                   double *partB, GridBarrier gb, int max_iter,
                                                                   double gap_tol, double *state,
                                                                   double *trace, int trace_cap,
                                                                   const __grid_constant__ CUtensorMap mapR,
                                                                   const __grid_constant__ CUtensorMap mapA,
                                                                   const __grid_constant__ CUtensorMap mapB,
                                                                   const __grid_constant__ CUtensorMap mapUi,
                                                                   const __grid_constant__ CUtensorMap mapRi) {
    __shared__ double sh[8];
    const size_t N = (size_t)W * H;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nthr = (size_t)gridDim.x * blockDim.x;
    __shared__ float tile[TMA ? 1 : 3][TMA ? 1 : kHaloY][TMA ? 1 : kHaloX];
    extern __shared__ __align__(128) float dyn_smem[];
    // TMA destinations: [stage][slot][kBoxStride], 128-byte aligned explicitly
    float *boxes = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(dyn_smem) + 127) & ~uintptr_t(127));
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_flag;
    unsigned par[2] = {0u, 0u};
    const int tiles_x = (W + kTileX - 1) / kTileX, ntiles = tiles_x * ((H + kTileY - 1) / kTileY);
    const int nk = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const float lambda = 1.0f;
    unsigned int gen = 0;
    if (TMA && threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_proxy_async_smem();
    }
    __syncthreads();
    // thread 0 starts the loads of this block's k-th tile into stage k & 1. Phase A: halo boxes of r and d_old
    // (slots 0, 1). Phase B: halo box of d_new (slot 0) and the interior boxes of u and r (slots 1, 2).
    auto slot = [&](int st, int j) { return boxes + (size_t)(3 * st + j) * kBoxStride; };
    auto issue = [&](int k, bool phase_b, const CUtensorMap *halo1) {
        if (threadIdx.x != 0) return;
        const int t = (int)blockIdx.x + k * (int)gridDim.x, st = k & 1;
        const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
        fence_proxy_async_smem();
        if (!phase_b) {
            mbar_arrive_expect_tx(&bars[st], 2 * kBoxBytes);
            tma_load_3d(slot(st, 0), &mapR, x0 - 4, y0 - 1, 0, &bars[st]);
            tma_load_3d(slot(st, 1), halo1, x0 - 4, y0 - 1, 0, &bars[st]);
        } else {
            mbar_arrive_expect_tx(&bars[st], kBoxBytes + 2 * kIntBytes);
            tma_load_3d(slot(st, 0), halo1, x0 - 4, y0 - 1, 0, &bars[st]);
            tma_load_3d(slot(st, 1), &mapUi, x0, y0, 0, &bars[st]);
            tma_load_3d(slot(st, 2), &mapRi, x0, y0, 0, &bars[st]);
        }
    };
    // on a box that never arrived: flag the error, give the other stage's load a bounded wait, leave
    auto abandon = [&](int k) {
        if (threadIdx.x == 0) {
            atomicExch(gb.err, 1);
            if (k + 1 < nk) mbar_wait(&bars[(k + 1) & 1], par[(k + 1) & 1], kSpinLimit);
        }
    };
    // ---- phase 0: r = b - A x (initConjGrad, solver.cu:383-467) and the energy F(x)
    {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (size_t o = tid; o < N; o += nthr) {
            cg_start_pixel(W, H, N, o, gX, gY, U, U0, r, lambda, acc);
        }
        block_partials_f(acc, 4, partB, gridDim.x);
    }
    if (TMA) fence_proxy_async_global();
    if (!grid_sync(gb, gen)) return;
    block_reduce_partials(partB, gridDim.x, 4, sh);
    // The FP64 scalars (delta, E, gap) live in thread 0 of each block, which derives the float coefficients
    // and the stop decision and hands them to the block through shared memory (every block computes the same
    // values from the same partials, so the grid agrees).
    __shared__ float s_coef[3];
    __shared__ int s_stop;
    double delta[3] = {sh[0], sh[1], sh[2]};
    double E = sh[3];
    float beta[3] = {0.f, 0.f, 0.f};
    const float *dold = r;  // d_0 = r_0 (beta = 0)
    float *dnew = dA;
    double gap = 1e300;
    int it = 0;
    for (;; ++it) {
        if (threadIdx.x == 0) {
            const double bound = (delta[0] + delta[1] + delta[2]) / (2.0 * (double)lambda);
            gap = (E - bound) > 0 ? bound / (E - bound) : 1e300;
            s_stop = (it >= max_iter || (gap_tol > 0 && gap <= gap_tol)) ? 1 : 0;
        }
        __syncthreads();
        if (s_stop) break;
        // ---- phase A: d = r + beta d_old on each tile + halo in shared memory, q = A d, d . q
        float accA[4] = {0.f, 0.f, 0.f, 0.f};
        if constexpr (TMA) {
            const CUtensorMap *mdold = (dold == r) ? &mapR : (dold == dA ? &mapA : &mapB);
            if (nk > 0) issue(0, false, mdold);
            for (int k = 0; k < nk; ++k) {
                if (k + 1 < nk) issue(k + 1, false, mdold);
                const int st = k & 1;
                if (!block_wait_box(&bars[st], par[st], &s_flag)) {
                    abandon(k);
                    return;
                }
                par[st] ^= 1u;
                const int t = (int)blockIdx.x + k * (int)gridDim.x;
                const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
                const float *R = slot(st, 0), *D = slot(st, 1);
                for (int p = threadIdx.x; p < kTileX * kTileY; p += blockDim.x) {
                    const int lx = p % kTileX, ly = p / kTileX, x = x0 + lx, y = y0 + ly;
                    if (x >= W || y >= H) continue;
                    const size_t o = (size_t)y * W + x;
                    const int bi = (ly + 1) * kBoxX + (lx + 4);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float *Rc = R + c * kBoxPlane, *Dc = D + c * kBoxPlane;
                        const float b = beta[c];
                        auto v = [&](int i) { return Rc[i] + b * Dc[i]; };
                        const float qv = box_op(v, bi, x, y, W, H, lambda);
                        const float dcv = v(bi);
                        dnew[c * N + o] = dcv;
                        accA[c] += dcv * qv;
                    }
                }
                __syncthreads();
            }
        } else {
            float *acc = accA;
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
                const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
                for (int k = threadIdx.x; k < 3 * kHaloY * kHaloX; k += blockDim.x) {
                    const int c = k / (kHaloY * kHaloX), rem = k % (kHaloY * kHaloX);
                    const int gx = x0 - 1 + rem % kHaloX, gy = y0 - 1 + rem / kHaloX;
                    float v = 0.f;
                    if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
                        const size_t o = c * N + (size_t)gy * W + gx;
                        v = __ldcg(r + o) + beta[c] * __ldcg(dold + o);
                    }
                    tile[c][rem / kHaloX][rem % kHaloX] = v;
                }
                __syncthreads();
                for (int p = threadIdx.x; p < kTileX * kTileY; p += blockDim.x) {
                    const int lx = p % kTileX, ly = p / kTileX, x = x0 + lx, y = y0 + ly;
                    if (x >= W || y >= H) continue;
                    const size_t o = (size_t)y * W + x;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float qv = tile_op(tile[c], lx + 1, ly + 1, x, y, W, H, lambda);
                        const float dcv = tile[c][ly + 1][lx + 1];
                        dnew[c * N + o] = dcv;
                        acc[c] += dcv * qv;
                    }
                }
                __syncthreads();
            }
        }
        block_partials_f(accA, 3, partA, gridDim.x);
        if (TMA) fence_proxy_async_global();
        if (!grid_sync(gb, gen)) return;
        block_reduce_partials(partA, gridDim.x, 3, sh);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double alpha_d = (sh[c] > 0) ? delta[c] / sh[c] : 0.0;
                s_coef[c] = (float)alpha_d;
                E -= 0.5 * alpha_d * delta[c];
            }
            if (blockIdx.x == 0 && trace && it < trace_cap) trace[it] = E;
        }
        __syncthreads();
        const float alpha[3] = {s_coef[0], s_coef[1], s_coef[2]};
        // ---- phase B: x += alpha d, r -= alpha A d, r . r (d tile + halo in shared memory)
        float accB[4] = {0.f, 0.f, 0.f, 0.f};
        if constexpr (TMA) {
            const CUtensorMap *mdnew = (dnew == dA) ? &mapA : &mapB;
            if (nk > 0) issue(0, true, mdnew);
            for (int k = 0; k < nk; ++k) {
                if (k + 1 < nk) issue(k + 1, true, mdnew);
                const int st = k & 1;
                if (!block_wait_box(&bars[st], par[st], &s_flag)) {
                    abandon(k);
                    return;
                }
                par[st] ^= 1u;
                const int t = (int)blockIdx.x + k * (int)gridDim.x;
                const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
                const float *Dn = slot(st, 0), *Ui = slot(st, 1), *Ri = slot(st, 2);
                for (int p = threadIdx.x; p < kTileX * kTileY; p += blockDim.x) {
                    const int lx = p % kTileX, ly = p / kTileX, x = x0 + lx, y = y0 + ly;
                    if (x >= W || y >= H) continue;
                    const size_t o = (size_t)y * W + x;
                    const int bi = (ly + 1) * kBoxX + (lx + 4);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float *Dc = Dn + c * kBoxPlane;
                        auto v = [&](int i) { return Dc[i]; };
                        const float qv = box_op(v, bi, x, y, W, H, lambda);
                        const float dv = Dc[bi];
                        U[c * N + o] = Ui[c * kTileX * kTileY + p] + alpha[c] * dv;
                        const float rv = Ri[c * kTileX * kTileY + p] - alpha[c] * qv;
                        r[c * N + o] = rv;
                        accB[c] += rv * rv;
                    }
                }
                __syncthreads();
            }
        } else {
            float *acc = accB;
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
                const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
                for (int k = threadIdx.x; k < 3 * kHaloY * kHaloX; k += blockDim.x) {
                    const int c = k / (kHaloY * kHaloX), rem = k % (kHaloY * kHaloX);
                    const int gx = x0 - 1 + rem % kHaloX, gy = y0 - 1 + rem / kHaloX;
                    tile[c][rem / kHaloX][rem % kHaloX] =
                        (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __ldcg(dnew + c * N + (size_t)gy * W + gx) : 0.f;
                }
                __syncthreads();
                for (int p = threadIdx.x; p < kTileX * kTileY; p += blockDim.x) {
                    const int lx = p % kTileX, ly = p / kTileX, x = x0 + lx, y = y0 + ly;
                    if (x >= W || y >= H) continue;
                    const size_t o = (size_t)y * W + x;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float qv = tile_op(tile[c], lx + 1, ly + 1, x, y, W, H, lambda);
                        const float dv = tile[c][ly + 1][lx + 1];
                        U[c * N + o] = __ldcg(U + c * N + o) + alpha[c] * dv;
                        const float rv = __ldcg(r + c * N + o) - alpha[c] * qv;
                        r[c * N + o] = rv;
                        acc[c] += rv * rv;
                    }
                }
                __syncthreads();
            }
        }
        block_partials_f(accB, 3, partB, gridDim.x);
        if (TMA) fence_proxy_async_global();
        if (!grid_sync(gb, gen)) return;
        block_reduce_partials(partB, gridDim.x, 3, sh);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                s_coef[c] = (delta[c] > 0) ? (float)(sh[c] / delta[c]) : 0.f;
                delta[c] = sh[c];
            }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 3; ++c) beta[c] = s_coef[c];
        dold = dnew;
        dnew = (dnew == dA) ? dB : dA;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        state[0] = delta[0];
        state[1] = delta[1];
        state[2] = delta[2];
        state[3] = E;
        state[4] = gap;
        state[5] = (double)it;
    }
}

// Shared-memory resident form of the corrected CG (the iteration of k_cg_persistent) for images of at most
// kResMaxTiles tiles per SM. Block b owns tiles b, b + G, ... and keeps r (3 planes) and d (3 planes with a
// one-pixel halo) of each in shared memory for the whole solve; only u stays in global memory. The phases
// exchange tile borders alone, through `bord` (set 0: r; sets 1, 2: d by iteration parity, since phase A still
// reads the previous iteration's d as d_old):
//   phase A: d = r + beta d_old on the interior; the halo's d from the neighbours' published r and d_old
//            borders; q = A d, d . q; publish the border rows and columns of d;
//   phase B: the halo's d from the neighbours' new borders; q = A d; u += alpha d; r -= alpha q, r . r;
//            publish the borders of r.
// Per pixel the arithmetic is k_cg_persistent's. Borders written by other blocks are read through L2 (__ldcg)
// after the grid barrier that follows their writing.
constexpr int kResThreads = kTileX * kTileY;          // one tile pixel per thread
constexpr int kResMaxTiles = 7;                       // tiles per block: 7 x 26.5 KB of shared memory
constexpr int kResPix = kTileX * kTileY;              // r plane (interior only)
constexpr int kResPlane = kHaloY * kHaloX;            // d plane with its halo: 18 x 66 floats
constexpr int kResBorder = 2 * kTileX + 2 * kTileY;   // border values per plane: top, bottom, left, right rows
constexpr size_t kResTileBytes = (size_t)3 * (kResPix + kResPlane) * sizeof(float);

// a / b in FP64 for the solver's scalars: an FP32 reciprocal refined by Newton steps in FP64 (a few dependent
// FMAs instead of the full division sequence, whose latency sits on the path every block waits for). The
// result is within a few units in the last place of the rounded quotient; b outside the FP32 range takes
// the division.
__device__ __forceinline__ double res_div(double a, double b) {
    const double ab = fabs(b);
    if (!(ab > 1e-30 && ab < 1e30)) return a / b;
    double r = (double)__frcp_rn((float)b);
    r = fma(r, fma(-b, r, 1.0), r);  // ~46 bits
    r = fma(r, fma(-b, r, 1.0), r);  // full precision
    const double q = a * r;
    return fma(r, fma(-b, q, a), q);
}

// Halo slot p (in [0, kResBorder)) of a tile at tile coordinates (tx, ty): its index in a d plane, and the
// neighbour tile and border slot it is read from (nt = -1: outside the image, the value is 0). Border slots:
// top row [0, 64), bottom row [64, 128), left column [128, 144), right column [144, 160).
__device__ __forceinline__ void res_halo_slot(int p, int t, int tx, int ty, int tiles_x, int tiles_y, int &si,
                                              int &nt, int &np) {
    nt = -1;
    np = 0;
    if (p < kTileX) {  // row above <- bottom row of the tile above
        si = p + 1;
        if (ty > 0) nt = t - tiles_x, np = kTileX + p;
    } else if (p < 2 * kTileX) {  // row below <- top row of the tile below
        const int q = p - kTileX;
        si = (kTileY + 1) * kHaloX + q + 1;
        if (ty + 1 < tiles_y) nt = t + tiles_x, np = q;
    } else if (p < 2 * kTileX + kTileY) {  // left column <- right column of the tile to the left
        const int q = p - 2 * kTileX;
        si = (q + 1) * kHaloX;
        if (tx > 0) nt = t - 1, np = 2 * kTileX + kTileY + q;
    } else {  // right column <- left column of the tile to the right
        const int q = p - 2 * kTileX - kTileY;
        si = (q + 1) * kHaloX + kHaloX - 1;
        if (tx + 1 < tiles_x) nt = t + 1, np = 2 * kTileX + q;
    }
}

__global__ void __launch_bounds__(kResThreads, 1) k_cg_resident(int W, int H, const float *__restrict__ gX,
                                                                const float *__restrict__ gY, float *__restrict__ U,
                                                                const float *__restrict__ U0,
                                                                float *__restrict__ bord, double *__restrict__ partA,
                                                                double *__restrict__ partB, GridBarrier gb,
                                                                int max_iter, double gap_tol,
                                                                double *__restrict__ state,
                                                                double *__restrict__ trace, int trace_cap) {
    extern __shared__ __align__(16) float res_smem[];
    __shared__ double sh[4], s_delta[3], s_dE[3];
    __shared__ float s_coef[3];
    __shared__ int s_stop;
    __shared__ int s_x0[kResMaxTiles], s_y0[kResMaxTiles], s_inner[kResMaxTiles];
    __shared__ short s_slotD[kResBorder], s_slotR[kResBorder];  // border slot -> index in a d / r plane
    const size_t N = (size_t)W * H;
    const int tiles_x = (W + kTileX - 1) / kTileX, tiles_y = (H + kTileY - 1) / kTileY, ntiles = tiles_x * tiles_y;
    const int nk = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int lx = threadIdx.x % kTileX, ly = threadIdx.x / kTileX;
    const int si = (ly + 1) * kHaloX + lx + 1;  // this thread's pixel in a d plane
    float *Rs = res_smem;                       // [tile][plane][kResPix]
    float *Ds = res_smem + (size_t)nk * 3 * kResPix;  // [tile][plane][kResPlane]
    const float lambda = 1.0f;
    unsigned int gen = 0;
    auto tile_of = [&](int k) { return (int)blockIdx.x + k * (int)gridDim.x; };
    auto border = [&](int set, int t, int c) { return bord + ((size_t)(set * ntiles + t) * 3 + c) * kResBorder; };
    if ((int)threadIdx.x < nk) {
        const int t = tile_of(threadIdx.x), x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
        s_x0[threadIdx.x] = x0;
        s_y0[threadIdx.x] = y0;
        // no pixel of an inner tile sits on the image border: its operator needs no one-sided differences
        s_inner[threadIdx.x] = (x0 > 0 && y0 > 0 && x0 + kTileX < W && y0 + kTileY < H) ? 1 : 0;
    }
    if ((int)threadIdx.x < kResBorder) {
        const int p = threadIdx.x;
        int px, py;  // tile pixel of border slot p
        if (p < kTileX) px = p, py = 0;
        else if (p < 2 * kTileX) px = p - kTileX, py = kTileY - 1;
        else if (p < 2 * kTileX + kTileY) px = 0, py = p - 2 * kTileX;
        else px = kTileX - 1, py = p - 2 * kTileX - kTileY;
        s_slotD[p] = (short)((py + 1) * kHaloX + px + 1);
        s_slotR[p] = (short)(py * kTileX + px);
    }
    __syncthreads();
    // Border values of every own tile, one (tile, plane, slot) item at a time: d from the interior of the
    // shared d planes (D = true) or r from the r planes, into border set `set`.
    // (item j = (k * 3 + c) * kResBorder + p lands at border(set, tile k, c)[p], i.e. at
    // bord + (set * ntiles + blockIdx.x) * 3 kResBorder + j + k (gridDim.x - 1) 3 kResBorder)
    auto publish = [&](int set, bool D) {
        float *base = bord + ((size_t)set * ntiles + blockIdx.x) * 3 * kResBorder;
        const size_t kstep = (size_t)(gridDim.x - 1) * 3 * kResBorder;
        for (int j = threadIdx.x; j < nk * 3 * kResBorder; j += kResThreads) {
            const int q = j / kResBorder, p = j - q * kResBorder, k = q / 3;  // q = k * 3 + c
            const float v = D ? Ds[q * kResPlane + s_slotD[p]] : Rs[q * kResPix + s_slotR[p]];
            base[j + k * kstep] = v;
        }
    };
    // Halo of every own tile's d planes from the neighbours' borders: border(sa) + b_c border(sb) (sb < 0:
    // border(sa) alone; 0 outside the image). load_halo issues all of a thread's loads into hv / hi,
    // store_halo writes them to the planes, so other work can run while the loads are in flight.
    constexpr int kItems = (kResMaxTiles * 3 * kResBorder + kResThreads - 1) / kResThreads;
    float hv[kItems];
    int hi[kItems];
    auto load_halo = [&](int sa, int sb, float b0, float b1, float b2) {
#pragma unroll
        for (int u = 0; u < kItems; ++u) {
            const int j = (int)threadIdx.x + u * kResThreads;
            hv[u] = 0.f;
            hi[u] = -1;
            if (j < nk * 3 * kResBorder) {
                const int k = j / (3 * kResBorder), rem = j - k * 3 * kResBorder, c = rem / kResBorder;
                const int t = tile_of(k);
                int hs, nt, np;
                res_halo_slot(rem - c * kResBorder, t, t % tiles_x, t / tiles_x, tiles_x, tiles_y, hs, nt, np);
                hi[u] = (k * 3 + c) * kResPlane + hs;
                if (nt >= 0) {
                    hv[u] = __ldcg(border(sa, nt, c) + np);
                    if (sb >= 0) hv[u] += (c == 0 ? b0 : (c == 1 ? b1 : b2)) * __ldcg(border(sb, nt, c) + np);
                }
            }
        }
    };
    auto store_halo = [&]() {
#pragma unroll
        for (int u = 0; u < kItems; ++u)
            if (hi[u] >= 0) Ds[hi[u]] = hv[u];
    };
    // q = A d at this thread's pixel of plane Dc (inner tiles: the interior formula of box_op, same arithmetic)
    auto op_at = [&](const float *Dc, bool inner, int x, int y) {
        if (inner) {
            const float c = Dc[si];
            const float lxv = 2.f * c - Dc[si - 1] - Dc[si + 1];
            const float lyv = 2.f * c - Dc[si - kHaloX] - Dc[si + kHaloX];
            return lambda * c + lxv + lyv;
        }
        return box_op<kHaloX>([&](int i) { return Dc[i]; }, si, x, y, W, H, lambda);
    };
    // ---- phase 0: r = b - A x and the energy F(x); d_old = 0 (interior and published borders)
    {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < nk; ++k) {
            const int x = s_x0[k] + lx, y = s_y0[k] + ly;
            float rv[3] = {0.f, 0.f, 0.f};
            if (x < W && y < H) cg_start_values(W, H, N, (size_t)y * W + x, x, y, gX, gY, U, U0, lambda, rv, acc);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                Rs[(k * 3 + c) * kResPix + threadIdx.x] = rv[c];
                Ds[(k * 3 + c) * kResPlane + si] = 0.f;
            }
        }
        __syncthreads();
        publish(0, false);
        publish(2, true);
        block_partials_f(acc, 4, partB, gridDim.x);
    }
    if (!grid_sync(gb, gen)) return;
    block_reduce_partials(partB, gridDim.x, 4, sh);
    if (threadIdx.x < 3) s_delta[threadIdx.x] = sh[threadIdx.x];
    double E = sh[3];  // thread 0's copy is the one in use
    float beta[3] = {0.f, 0.f, 0.f};
    int it = 0;
    __syncthreads();
    for (;; ++it) {
        if (threadIdx.x == 0) {
            // gap = bound / (E - bound) <= gap_tol, tested without the division
            const double bound = (s_delta[0] + s_delta[1] + s_delta[2]) / (2.0 * (double)lambda);
            const double room = E - bound;
            s_stop = (it >= max_iter || (gap_tol > 0 && room > 0 && bound <= gap_tol * room)) ? 1 : 0;
        }
        __syncthreads();
        if (s_stop) break;
        const int dold = 1 + ((it + 1) & 1), dnew = 1 + (it & 1);
        // ---- phase A: d = r + beta d_old (halo from the neighbours' borders, interior in place); publish d's
        // borders; q = A d and d . q
        load_halo(0, dold, beta[0], beta[1], beta[2]);
        for (int k = 0; k < nk; ++k)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float *d = Ds + (k * 3 + c) * kResPlane + si;
                *d = Rs[(k * 3 + c) * kResPix + threadIdx.x] + beta[c] * *d;
            }
        store_halo();
        __syncthreads();
        publish(dnew, true);
        float accA[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < nk; ++k) {
            const int x = s_x0[k] + lx, y = s_y0[k] + ly;
            if (x >= W || y >= H) continue;
            const bool inner = s_inner[k] != 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float *Dc = Ds + (k * 3 + c) * kResPlane;
                accA[c] += Dc[si] * op_at(Dc, inner, x, y);
            }
        }
        block_partials_f(accA, 3, partA, gridDim.x);
        if (!grid_sync(gb, gen)) return;
        block_reduce_partials(partA, gridDim.x, 3, sh);
        // the three step lengths on three threads (the FP64 divisions side by side)
        if (threadIdx.x < 3) {
            const int c = threadIdx.x;
            const double alpha_d = (sh[c] > 0) ? res_div(s_delta[c], sh[c]) : 0.0;
            s_coef[c] = (float)alpha_d;
            s_dE[c] = 0.5 * alpha_d * s_delta[c];
        }
        __syncthreads();
        const float alpha[3] = {s_coef[0], s_coef[1], s_coef[2]};
        if (threadIdx.x == 0) {
            E = E - s_dE[0] - s_dE[1] - s_dE[2];
            if (blockIdx.x == 0 && trace && it < trace_cap) trace[it] = E;
        }
        // ---- phase B: the halo's d from the neighbours' new borders; u += alpha d, r -= alpha A d, r . r;
        // publish r's borders
        load_halo(dnew, -1, 0.f, 0.f, 0.f);
        store_halo();
        __syncthreads();
        float accB[4] = {0.f, 0.f, 0.f, 0.f};
        // u of the next tile is loaded while the current one is updated
        auto load_u = [&](int k, float u3[3]) {
            const int x = s_x0[k] + lx, y = s_y0[k] + ly;
            const bool in = x < W && y < H;
            const size_t o = (size_t)y * W + x;
#pragma unroll
            for (int c = 0; c < 3; ++c) u3[c] = in ? __ldcg(U + c * N + o) : 0.f;
        };
        float ucur[3] = {0.f, 0.f, 0.f};
        if (nk > 0) load_u(0, ucur);
        for (int k = 0; k < nk; ++k) {
            float unext[3] = {0.f, 0.f, 0.f};
            if (k + 1 < nk) load_u(k + 1, unext);
            const int x = s_x0[k] + lx, y = s_y0[k] + ly;
            if (x < W && y < H) {
                const bool inner = s_inner[k] != 0;
                const size_t o = (size_t)y * W + x;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float *Dc = Ds + (k * 3 + c) * kResPlane;
                    float *Rc = Rs + (k * 3 + c) * kResPix + threadIdx.x;
                    const float qv = op_at(Dc, inner, x, y);
                    U[c * N + o] = ucur[c] + alpha[c] * Dc[si];
                    const float rv = *Rc - alpha[c] * qv;
                    *Rc = rv;
                    accB[c] += rv * rv;
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) ucur[c] = unext[c];
        }
        __syncthreads();
        publish(0, false);
        block_partials_f(accB, 3, partB, gridDim.x);
        if (!grid_sync(gb, gen)) return;
        block_reduce_partials(partB, gridDim.x, 3, sh);
        if (threadIdx.x < 3) {
            const int c = threadIdx.x;
            s_coef[c] = (s_delta[c] > 0) ? (float)res_div(sh[c], s_delta[c]) : 0.f;
            s_delta[c] = sh[c];
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 3; ++c) beta[c] = s_coef[c];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double bound = (s_delta[0] + s_delta[1] + s_delta[2]) / (2.0 * (double)lambda);
        state[0] = s_delta[0];
        state[1] = s_delta[1];
        state[2] = s_delta[2];
        state[3] = E;
        state[4] = (E - bound) > 0 ? bound / (E - bound) : 1e300;
        state[5] = (double)it;
    }
}

// Batched corrected CG: many targets (CgProblem) in one cooperative launch. Each problem owns the blocks
// [b0, b0 + nb) (block_prob maps a block to its problem), so its tiles, block partials and FP64 scalars never mix
// with another problem's; all problems share the grid barriers. A problem that has met its stop rule idles;
// done[p] (written by the problem's first block at the top of every iteration) tells every block, after the next
// barrier, whether all problems have stopped, and then the whole grid leaves together. Per problem the
// arithmetic is k_cg_persistent<false>'s.
__global__ void __launch_bounds__(kPersistThreads) k_cg_batch(const CgProblem *__restrict__ probs,
                                                              const int *__restrict__ block_prob, int nprob,
                                                              double *partA, double *partB, int *done,
                                                              GridBarrier gb) {
    __shared__ double sh[8];
    __shared__ float tile[3][kHaloY][kHaloX];
    __shared__ float s_coef[3];
    __shared__ int s_stop, s_all;
    const int pid = block_prob[blockIdx.x];
    const CgProblem P = probs[pid];
    const int W = P.W, H = P.H;
    const size_t N = (size_t)W * H;
    const int lb = (int)blockIdx.x - P.b0;  // block index within the problem
    const int G = (int)gridDim.x;
    const float lambda = 1.0f;
    float *U = P.U, *r = P.r;
    unsigned int gen = 0;
    // ---- phase 0 (as k_cg_persistent): r = b - A x and F(x)
    {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (size_t o = (size_t)lb * blockDim.x + threadIdx.x; o < N; o += (size_t)P.nb * blockDim.x) {
            cg_start_pixel(W, H, N, o, P.gx, P.gy, U, P.U0, r, lambda, acc);
        }
        block_partials_f(acc, 4, partB, G);
    }
    if (!grid_sync(gb, gen)) return;
    // the problem's partials sit at [slot * G + b0, slot * G + b0 + nb): one warp per slot sums them in a fixed order
    auto reduce_own = [&](const double *part, int nslots) { reduce_slots(part + P.b0, P.nb, (size_t)G, nslots, sh); };
    reduce_own(partB, 4);
    double delta[3] = {sh[0], sh[1], sh[2]};
    double E = sh[3];
    double gap = 1e300;
    float beta[3] = {0.f, 0.f, 0.f};
    const float *dold = r;
    float *dnew = P.dA;
    int it = 0, stopped_at = -1;
    const int tiles_x = P.tiles_x, ntiles = P.ntiles;
    for (;; ++it) {
        if (threadIdx.x == 0) {
            if (stopped_at < 0) {
                const double bound = (delta[0] + delta[1] + delta[2]) / (2.0 * (double)lambda);
                gap = (E - bound) > 0 ? bound / (E - bound) : 1e300;
                if (it >= P.max_iter || (P.gap_tol > 0 && gap <= P.gap_tol)) stopped_at = it;
            }
            s_stop = stopped_at >= 0 ? 1 : 0;
            if (lb == 0) done[pid] = s_stop;
        }
        __syncthreads();
        const bool idle = s_stop != 0;
        // ---- phase A (skipped by a stopped problem)
        {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            if (!idle) {
                for (int t = lb; t < ntiles; t += P.nb) {
                    const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
                    for (int k = threadIdx.x; k < 3 * kHaloY * kHaloX; k += blockDim.x) {
                        const int c = k / (kHaloY * kHaloX), rem = k % (kHaloY * kHaloX);
                        const int gx = x0 - 1 + rem % kHaloX, gy = y0 - 1 + rem / kHaloX;
                        float v = 0.f;
                        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
                            const size_t o = c * N + (size_t)gy * W + gx;
                            v = __ldcg(r + o) + beta[c] * __ldcg(dold + o);
                        }
                        tile[c][rem / kHaloX][rem % kHaloX] = v;
                    }
                    __syncthreads();
                    for (int p = threadIdx.x; p < kTileX * kTileY; p += blockDim.x) {
                        const int lx = p % kTileX, ly = p / kTileX, x = x0 + lx, y = y0 + ly;
                        if (x >= W || y >= H) continue;
                        const size_t o = (size_t)y * W + x;
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const float qv = tile_op(tile[c], lx + 1, ly + 1, x, y, W, H, lambda);
                            const float dcv = tile[c][ly + 1][lx + 1];
                            dnew[c * N + o] = dcv;
                            acc[c] += dcv * qv;
                        }
                    }
                    __syncthreads();
                }
            }
            block_partials_f(acc, 3, partA, G);
        }
        if (!grid_sync(gb, gen)) return;
        // every problem wrote done[] before this barrier: leave together once all have stopped
        if (threadIdx.x == 0) {
            int all = 1;
            for (int q = 0; q < nprob; ++q) all &= __ldcg(done + q);
            s_all = all;
        }
        __syncthreads();
        if (s_all) break;
        if (!idle) reduce_own(partA, 3);
        if (threadIdx.x == 0 && !idle) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double alpha_d = (sh[c] > 0) ? delta[c] / sh[c] : 0.0;
                s_coef[c] = (float)alpha_d;
                E -= 0.5 * alpha_d * delta[c];
            }
            if (lb == 0 && P.trace && it < P.trace_cap) P.trace[it] = E;
        }
        __syncthreads();
        const float alpha[3] = {s_coef[0], s_coef[1], s_coef[2]};
        // ---- phase B
        {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            if (!idle) {
                for (int t = lb; t < ntiles; t += P.nb) {
                    const int x0 = (t % tiles_x) * kTileX, y0 = (t / tiles_x) * kTileY;
                    for (int k = threadIdx.x; k < 3 * kHaloY * kHaloX; k += blockDim.x) {
                        const int c = k / (kHaloY * kHaloX), rem = k % (kHaloY * kHaloX);
                        const int gx = x0 - 1 + rem % kHaloX, gy = y0 - 1 + rem / kHaloX;
                        tile[c][rem / kHaloX][rem % kHaloX] =
                            (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __ldcg(dnew + c * N + (size_t)gy * W + gx) : 0.f;
                    }
                    __syncthreads();
                    for (int p = threadIdx.x; p < kTileX * kTileY; p += blockDim.x) {
                        const int lx = p % kTileX, ly = p / kTileX, x = x0 + lx, y = y0 + ly;
                        if (x >= W || y >= H) continue;
                        const size_t o = (size_t)y * W + x;
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const float qv = tile_op(tile[c], lx + 1, ly + 1, x, y, W, H, lambda);
                            const float dv = tile[c][ly + 1][lx + 1];
                            U[c * N + o] = __ldcg(U + c * N + o) + alpha[c] * dv;
                            const float rv = __ldcg(r + c * N + o) - alpha[c] * qv;
                            r[c * N + o] = rv;
                            acc[c] += rv * rv;
                        }
                    }
                    __syncthreads();
                }
            }
            block_partials_f(acc, 3, partB, G);
        }
        if (!grid_sync(gb, gen)) return;
        if (!idle) {
            reduce_own(partB, 3);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    s_coef[c] = (delta[c] > 0) ? (float)(sh[c] / delta[c]) : 0.f;
                    delta[c] = sh[c];
                }
            }
            __syncthreads();
#pragma unroll
            for (int c = 0; c < 3; ++c) beta[c] = s_coef[c];
            dold = dnew;
            dnew = (dnew == P.dA) ? P.dB : P.dA;
        }
    }
    if (lb == 0 && threadIdx.x == 0) {
        P.state[0] = delta[0];
        P.state[1] = delta[1];
        P.state[2] = delta[2];
        P.state[3] = E;
        P.state[4] = gap;
        P.state[5] = (double)(stopped_at >= 0 ? stopped_at : it);
    }
}

// Hole filling in shared memory, without a grid barrier: one block (C = 1) for at most kSmallHoles holes, or one
// cluster of C blocks for at most C * kSmallHoles, each block holding a contiguous share of the sorted hole list.
// The visible pixels never change, so every hole keeps, per direction (left, up, right, down: the summation order
// of compute_laplacian), either a reference to the neighbouring hole (block rank << 11 | index in that block's
// share) or the neighbour's fixed value; the iterations then touch shared memory only, a cluster's blocks reading
// each other's shares through distributed shared memory, with one cluster barrier per iteration. Each update
// gives k_hole_fill_persistent's value bit for bit (its division by the neighbour count is a corrected
// reciprocal product). holes must be in ascending pixel order with the row starts behind them (launch_hole_list).
constexpr int kSmallHoles = 2048, kSmallThreads = 1024, kHoleCluster = 8;
static_assert(kSmallHoles == 1 << 11 && kHoleCluster * kSmallHoles <= 32767, "hole references are 16-bit");
constexpr size_t kSmallHoleSmem = (size_t)kSmallHoles * (6 * 4 + 12 * 4 + 4 * 2 + 4);

template <int C>
__global__ void __launch_bounds__(kSmallThreads) k_hole_fill_small(int W, int H, const int *__restrict__ holes,
                                                                   const int *__restrict__ count, float *A,
                                                                   int max_iter, double *state) {
    const int nh = *count;
    // the sizes this form takes (every block of a cluster returns together, before any cluster barrier)
    if (nh > C * kSmallHoles || (C > 1 && nh <= kSmallHoles)) return;
    extern __shared__ __align__(16) float hsm[];
    float *cur = hsm, *nxt = hsm + 3 * kSmallHoles;            // [3][kSmallHoles] each
    float *fixedv = hsm + 6 * kSmallHoles;                      // [4 dirs][3][kSmallHoles]
    float *wts = hsm + 18 * kSmallHoles;                        // [kSmallHoles]
    __shared__ float rws[kSmallHoles];                          // 1 / wts
    short *nb = reinterpret_cast<short *>(hsm + 19 * kSmallHoles);  // [4][kSmallHoles]: reference, -1 fixed, -2 none
    __shared__ float wsum[2][kSmallThreads / 32];
    __shared__ int s_holes[kSmallHoles];
    const int rank = C > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int chunk = (nh + C - 1) / C, h0 = rank * chunk, nloc = max(0, min(nh - h0, chunk));
    const size_t N = (size_t)W * H;
    for (int h = threadIdx.x; h < nloc; h += kSmallThreads) s_holes[h] = __ldg(holes + h0 + h);
    __syncthreads();
    // row starts of the hole list (launch_hole_list keeps them in holes[N .. N + H)): a vertical neighbour is
    // searched in its row's few holes only, a horizontal one is the adjacent entry of the sorted list
    const int *row_start = holes + N;
    for (int h = threadIdx.x; h < nloc; h += kSmallThreads) {
        const int g = h0 + h, o = s_holes[h];
        const int ox = o % W, oy = o / W;
        const bool has[4] = {ox > 0, oy > 0, ox < W - 1, oy < H - 1};
        const int q[4] = {o - 1, o - W, o + 1, o + W};
        int lo[4] = {g - 1, 0, g + 1, 0}, hi[4] = {g - 1, -1, min(g + 1, nh - 1), -1};
        if (has[1]) {
            lo[1] = __ldg(row_start + oy - 1);
            hi[1] = __ldg(row_start + oy) - 1;
        }
        if (has[3]) {
            lo[3] = __ldg(row_start + oy + 1);
            hi[3] = (oy + 2 < H ? __ldg(row_start + oy + 2) : nh) - 1;
        }
        float wt = 0.f;
        short idx4[4];
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            short idx = -2;
            if (has[d]) {
                wt += 1.f;
                idx = -1;
                int l = max(lo[d], 0), r = hi[d];
                while (l <= r) {
                    const int mid = (l + r) >> 1, v = __ldg(holes + mid);
                    if (v == q[d]) {
                        const int rr = mid / chunk;
                        idx = (short)((rr << 11) | (mid - rr * chunk));
                        break;
                    }
                    if (v < q[d]) l = mid + 1;
                    else r = mid - 1;
                }
            }
            idx4[d] = idx;
            nb[d * kSmallHoles + h] = idx;
        }
        wts[h] = wt;
        rws[h] = 1.0f / wt;
        // the fixed neighbours' values and the hole's own, all loads issued together
#pragma unroll
        for (int d = 0; d < 4; ++d)
            if (idx4[d] == -1)
                for (int c = 0; c < 3; ++c) fixedv[(d * 3 + c) * kSmallHoles + h] = A[c * N + q[d]];
        for (int c = 0; c < 3; ++c) cur[c * kSmallHoles + h] = A[c * N + o];
    }
    // a cluster: every block's share is in place before any block reads another's
    if constexpr (C > 1) cg::this_cluster().sync();
    else __syncthreads();
    // one block: only the warps that hold holes iterate (at least one, so that an empty hole set reports its one
    // iteration as the reference does); the others leave, and the iterations synchronise on named barrier 1 with
    // the iterating threads' count. A cluster: every thread takes part in the cluster barriers.
    const int active = C > 1 ? kSmallThreads : max(32, min(kSmallThreads, (nloc + 31) & ~31));
    if ((int)threadIdx.x >= active) return;
    float energy = 0.0f, previous = 0.0f;
    int k;
    for (k = 0; k < max_iter; ++k) {
        previous = energy;
        // the energy in FP32 (a handful of terms per thread, fixed shuffle trees): the FP64 pipe of this part is
        // narrow, and the stop test compares single-precision energies
        float acc = 0.f;
        for (int h = threadIdx.x; h < nloc; h += kSmallThreads) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v = 0.f;
#pragma unroll
                for (int d = 0; d < 4; ++d) {
                    const short idx = nb[d * kSmallHoles + h];
                    if (idx == -2) continue;
                    if (idx == -1) {
                        v += fixedv[(d * 3 + c) * kSmallHoles + h];
                    } else {
                        const int rr = idx >> 11, l = idx & (kSmallHoles - 1);
                        const float *src = cur + c * kSmallHoles + l;
                        if constexpr (C > 1)
                            if (rr != rank) src = cg::this_cluster().map_shared_rank(src, rr);
                        v += *src;
                    }
                }
                // v / wt as the reciprocal product with one residual correction (Markstein): with rw the
                // rounded reciprocal and q within an ulp of the quotient, q + rw (v - wt q) is the correctly
                // rounded quotient, i.e. the division's result bit for bit (no underflow at these magnitudes)
                {
                    const float wt = wts[h], rw = rws[h];
                    const float q = v * rw;
                    v = fmaf(fmaf(-q, wt, v), rw, q);
                }
                const float uc = cur[c * kSmallHoles + h];
                const float lap = v - uc;
                const float un = uc + lap;
                nxt[c * kSmallHoles + h] = un;
                if (c == 2) acc += lap * un;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        // one barrier per iteration: the warp sums alternate between two slots, and every warp sums the 32 of
        // this iteration (of each block in rank order) with the same fixed tree, so all agree
        const int lane = threadIdx.x & 31;
        if (lane == 0) wsum[k & 1][threadIdx.x >> 5] = acc;
        float tot;
        if constexpr (C > 1) {
            cg::this_cluster().sync();
            tot = 0.f;
            for (int rr = 0; rr < C; ++rr) {
                const float *ws = cg::this_cluster().map_shared_rank(&wsum[k & 1][0], rr);
                float t = ws[lane];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
                tot += __shfl_sync(0xffffffffu, t, 0);
            }
        } else {
            asm volatile("bar.sync 1, %0;" ::"r"(active) : "memory");
            tot = (lane < active / 32) ? wsum[k & 1][lane] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
        }
        energy = __shfl_sync(0xffffffffu, tot, 0);
        float *t = cur;
        cur = nxt;
        nxt = t;
        if (fabsf(previous - energy) < 1e-3f) {
            ++k;
            break;
        }
    }
    for (int h = threadIdx.x; h < nloc; h += kSmallThreads) {
        const int o = s_holes[h];
#pragma unroll
        for (int c = 0; c < 3; ++c) A[c * N + o] = cur[c * kSmallHoles + h];
    }
    if (rank == 0 && threadIdx.x == 0) state[0] = (double)k;
    // no block leaves while another may still read its shared memory
    if constexpr (C > 1) cg::this_cluster().sync();
}

// Hole filling with the whole iteration loop in one launch (hole_filling, sources/gradientIBR.cu:87-152).
// count: device pointer to the number of holes. A holds the initial image (and the result); B is scratch, into
// which the kernel first copies every hole's value and its neighbours' (the pixels the iterations read).
// state: [0] iterations.
// Only as many blocks as the hole count needs take part (kHoleFillPerBlock holes each; the others return at
// once), so the grid barrier of each iteration spans few blocks, and none is needed when one block suffices. The energy partials alternate between two
// slots by iteration parity: a block overwrites slot k & 1 in iteration k + 2 only after every block passed
// the barrier of iteration k + 1, i.e. after all of them read it, so one barrier per iteration suffices.
constexpr int kHoleFillPerBlock = 4 * kPersistThreads;

__global__ void __launch_bounds__(kPersistThreads) k_hole_fill_persistent(int W, int H, const int *__restrict__ holes,
                                                                          const int *__restrict__ count, float *A,
                                                                          float *B, double *part, GridBarrier gb,
                                                                          int max_iter, double *state, int handled) {
    __shared__ double sh[8];
    const size_t N = (size_t)W * H;
    const int nh = *count;
    if (nh <= handled) return;  // k_hole_fill_small (one block or one cluster) has done it
    const int active = min((int)gridDim.x, max(1, (nh + kHoleFillPerBlock - 1) / kHoleFillPerBlock));
    if ((int)blockIdx.x >= active) return;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = active * blockDim.x;
    unsigned int gen = 0;
    // B = A at the holes and their neighbours; every copy of one pixel writes the same value
    for (int h = tid; h < nh; h += nthr) {
        const int o = __ldg(holes + h);
        const int ox = o % W, oy = o / W;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const size_t p = (size_t)c * N + o;
            B[p] = __ldcg(A + p);
            if (ox > 0) B[p - 1] = __ldcg(A + p - 1);
            if (oy > 0) B[p - W] = __ldcg(A + p - W);
            if (ox < W - 1) B[p + 1] = __ldcg(A + p + 1);
            if (oy < H - 1) B[p + W] = __ldcg(A + p + W);
        }
    }
    if (active > 1) {
        if (!grid_sync(gb, gen, active)) return;
    } else {
        __syncthreads();
    }
    float *src = A, *dst = B;
    float energy = 0.0f, previous = 0.0f;
    int k;
    for (k = 0; k < max_iter; ++k) {
        previous = energy;
        double acc[4] = {0, 0, 0, 0};
        for (int h = tid; h < nh; h += nthr) {
            const int o = __ldg(holes + h);
            const int ox = o % W, oy = o / W;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float *u = src + c * N;
                float v = 0.f, wt = 0.f;
                if (ox > 0) { v += __ldcg(u + o - 1); wt += 1.f; }
                if (oy > 0) { v += __ldcg(u + o - W); wt += 1.f; }
                if (ox < W - 1) { v += __ldcg(u + o + 1); wt += 1.f; }
                if (oy < H - 1) { v += __ldcg(u + o + W); wt += 1.f; }
                v /= wt;
                const float uc = __ldcg(u + o);
                const float lap = v - uc;
                const float un = uc + lap;
                dst[c * N + o] = un;
                if (c == 2) acc[0] += (double)(lap * un);
            }
        }
        double *slot = part + (size_t)(k & 1) * active;
        block_partials(acc, 1, slot, active);
        if (active > 1) {
            if (!grid_sync(gb, gen, active)) return;
        } else {
            __syncthreads();  // one block: its own global writes are visible to it after the block barrier
        }
        block_reduce_partials(slot, active, 1, sh);
        energy = (float)sh[0];
        float *t = src;
        src = dst;
        dst = t;
        if (fabsf(previous - energy) < 1e-3f) {
            ++k;
            break;
        }
    }
    if (src != A) {  // copy the holes of the result back into A
        for (int h = tid; h < nh; h += nthr) {
            const int o = __ldg(holes + h);
#pragma unroll
            for (int c = 0; c < 3; ++c) A[c * N + o] = __ldcg(src + c * N + o);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) state[0] = (double)k;
}

// ------------------------------------------------------------------ Jacobi Poisson integration
// poisson_jacobi (sources/gradientIBR.cu:923-1013): z = (m u0 - div g) / (4 + m) per channel (compute_divergence,
// jacobi_z, sources/gradientIBR_kernels.cuh:553-598), then sweeps x <- (x_l + x_u + x_r + x_d) / (4 + m) + z with the
// border pixel standing in for a missing neighbour (jacobi_B :600-643). The reference launches 2 kernels per channel
// and sweep; here one cooperative launch runs every sweep of all three channels, kJacK sweeps per grid barrier: a
// block stages its tile with a halo of kJacK pixels in shared memory (each sweep's stencil reaches one pixel) and
// ping-pongs there. Every operation is the reference's float expression in its order, without contraction.
constexpr int kJacTX = 32, kJacTY = 16, kJacK = 4, kJacThreads = 512;
constexpr int kJacRX = kJacTX + 2 * kJacK, kJacRY = kJacTY + 2 * kJacK, kJacRN = kJacRX * kJacRY;
constexpr size_t kJacSmem = (size_t)10 * kJacRN * sizeof(float);  // x (3 channels x 2 buffers), z (3), 4 + m

__global__ void k_jacobi_setup(int W, int H, const float *__restrict__ gX, const float *__restrict__ gY,
                               const float *__restrict__ mask, const float *__restrict__ U, float *__restrict__ z,
                               float *__restrict__ den) {
    const int ox = blockIdx.x * blockDim.x + threadIdx.x, oy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ox >= W || oy >= H) return;
    const size_t o = (size_t)oy * W + ox, N = (size_t)W * H;
    float dv = 0.0f;
    if (ox != 0 && ox != W - 1) dv = __fadd_rn(dv, __fsub_rn(gX[o + 1], gX[o - 1]) / 2);
    if (oy != 0 && oy != H - 1) dv = __fadd_rn(dv, __fsub_rn(gY[o + W], gY[o - W]) / 2);
    const float data_w = __fmul_rn(1.0f, mask[o]);
    const float d = __fadd_rn(4.0f, data_w);
    den[o] = d;
#pragma unroll
    for (int c = 0; c < 3; ++c) z[c * N + o] = __fsub_rn(__fmul_rn(data_w, U[c * N + o]), dv) / d;
}

__global__ void __launch_bounds__(kJacThreads) k_jacobi_persistent(int W, int H, int iters,
                                                                   const float *__restrict__ z,
                                                                   const float *__restrict__ den, float *U0, float *U1,
                                                                   GridBarrier gb) {
    extern __shared__ float jsm[];
    float *sX = jsm, *sZ = jsm + 6 * kJacRN, *sD = jsm + 9 * kJacRN;  // sX: [buffer][channel][kJacRN]
    const int tiles_x = (W + kJacTX - 1) / kJacTX, ntiles = tiles_x * ((H + kJacTY - 1) / kJacTY);
    const size_t N = (size_t)W * H;
    unsigned int gen = 0;
    int step = 0;
    for (int done = 0; done < iters; done += kJacK, ++step) {
        const int n_it = min(kJacK, iters - done);
        const float *Ui = (step & 1) ? U1 : U0;
        float *Uo = (step & 1) ? U0 : U1;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int rx0 = (t % tiles_x) * kJacTX - kJacK, ry0 = (t / tiles_x) * kJacTY - kJacK;
            for (int i = threadIdx.x; i < kJacRN; i += kJacThreads) {
                const int gx = rx0 + i % kJacRX, gy = ry0 + i / kJacRX;
                const bool in = gx >= 0 && gx < W && gy >= 0 && gy < H;
                const size_t o = in ? (size_t)gy * W + gx : 0;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    sX[c * kJacRN + i] = in ? __ldcg(Ui + c * N + o) : 0.f;
                    sZ[c * kJacRN + i] = in ? __ldg(z + c * N + o) : 0.f;
                }
                sD[i] = in ? __ldg(den + o) : 1.f;
            }
            __syncthreads();
            for (int it = 0; it < n_it; ++it) {
                const float *src = sX + (it & 1) * 3 * kJacRN;
                float *dst = sX + ((it + 1) & 1) * 3 * kJacRN;
                for (int i = threadIdx.x; i < kJacRN; i += kJacThreads) {
                    const int lx = i % kJacRX, ly = i / kJacRX, gx = rx0 + lx, gy = ry0 + ly;
                    if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float *x = src + c * kJacRN;
                        const float xc = x[i];
                        // neighbours outside the staged region are stale only where the tile does not look
                        const float xl = gx == 0 ? xc : (lx > 0 ? x[i - 1] : 0.f);
                        const float xu = gy == 0 ? xc : (ly > 0 ? x[i - kJacRX] : 0.f);
                        const float xr = gx == W - 1 ? xc : (lx + 1 < kJacRX ? x[i + 1] : 0.f);
                        const float xd = gy == H - 1 ? xc : (ly + 1 < kJacRY ? x[i + kJacRX] : 0.f);
                        float v = 0.0f;
                        v = __fadd_rn(v, xl);
                        v = __fadd_rn(v, xu);
                        v = __fadd_rn(v, xr);
                        v = __fadd_rn(v, xd);
                        v = v / sD[i];
                        dst[c * kJacRN + i] = __fadd_rn(v, sZ[c * kJacRN + i]);
                    }
                }
                __syncthreads();
            }
            const float *res = sX + (n_it & 1) * 3 * kJacRN;
            for (int i = threadIdx.x; i < kJacTX * kJacTY; i += kJacThreads) {
                const int lx = kJacK + i % kJacTX, ly = kJacK + i / kJacTX, gx = rx0 + lx, gy = ry0 + ly;
                if (gx >= W || gy >= H) continue;
                const size_t o = (size_t)gy * W + gx;
                const int r = ly * kJacRX + lx;
#pragma unroll
                for (int c = 0; c < 3; ++c) Uo[c * N + o] = res[c * kJacRN + r];
            }
            __syncthreads();  // the next tile overwrites the staged region
        }
        if (!grid_sync(gb, gen)) return;
    }
}

// ------------------------------------------------------------------ launchers
static inline dim3 cg_grid(int W, int H) { return dim3((W + kCgBX - 1) / kCgBX, (H + kCgBY - 1) / kCgBY); }
int cg_partials(int W, int H) {
    const dim3 g = cg_grid(W, H);
    return (int)(g.x * g.y);
}

void launch_hole_list(int W, int H, const uint8_t *vis, int *holes, int *count, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "hole_list", st);
    // row starts are kept in holes[N .. N + H) scratch supplied by the caller (holes has N + H entries)
    int *row = holes + (size_t)W * H;
    const int rows_per_block = 256 / 32;
    // programmatic launches: each kernel's launch overlaps the tail of the one before it
    const dim3 rows_grid((H + rows_per_block - 1) / rows_per_block);
    launch_pdl(k_hole_rows, rows_grid, dim3(256), 0, st, W, H, vis, row);
    launch_pdl(k_hole_scan, dim3(1), dim3(1024), 0, st, H, row, count);
    launch_pdl(k_hole_write, rows_grid, dim3(256), 0, st, W, H, vis, row, holes);
    lc.add(3);
}

int hole_fill_partials(int nholes) { return (nholes + 255) / 256; }

// Blocks of a cooperative launch: every block must be resident at once (the grid barrier waits for all).
static int coop_blocks(const void *kernel, int want, size_t smem = 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistThreads, smem);
    per_sm = per_sm < 2 ? per_sm : 2;
    const int resident = sms * per_sm;
    return want < resident ? (want > 0 ? want : 1) : resident;
}

int persistent_partials() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return 2 * sms;
}

cudaError_t launch_poisson_jacobi(int W, int H, int iters, const float *gx, const float *gy, const float *mask,
                                  float *U, float *U1, float *z, float *den, GridBarrier gb, cudaStream_t st,
                                  LaunchCounter &lc) {
    ProfScope _ps(lc, "poisson_jacobi", st);
    const dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
    k_jacobi_setup<<<g, b, 0, st>>>(W, H, gx, gy, mask, U, z, den);
    lc.add(1);
    if (iters <= 0) return cudaGetLastError();
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi_persistent, kJacThreads, kJacSmem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int ntiles = ((W + kJacTX - 1) / kJacTX) * ((H + kJacTY - 1) / kJacTY);
    const int resident = sms * per_sm;
    const int per_block = (ntiles + resident - 1) / resident;
    const int blocks = std::max(1, (ntiles + per_block - 1) / per_block);
    void *args[] = {&W, &H, &iters, (void *)&z, (void *)&den, &U, &U1, &gb};
    e = cudaLaunchCooperativeKernel((const void *)k_jacobi_persistent, dim3(blocks), dim3(kJacThreads), args, kJacSmem,
                                    st);
    lc.add(1);
    if (e != cudaSuccess) return e;
    // an odd number of super-steps leaves the result in U1
    const int steps = (iters + kJacK - 1) / kJacK;
    if (steps & 1) return cudaMemcpyAsync(U, U1, sizeof(float) * 3 * (size_t)W * H, cudaMemcpyDeviceToDevice, st);
    return cudaSuccess;
}

cudaError_t launch_cg_persistent(int W, int H, const float *gx, const float *gy, float *U, float *r, float *dA,
                                 float *dB, double *partA, double *partB, GridBarrier gb, int max_iter, double gap_tol,
                                 double *state, cudaStream_t st, LaunchCounter &lc, const float *U0,
                                 double *trace, int trace_cap) {
    ProfScope _ps(lc, "cg_persistent", st);
    const size_t N = (size_t)W * H;
    const int ntiles = ((W + kTileX - 1) / kTileX) * ((H + kTileY - 1) / kTileY);
    // shared-memory resident form when every block can hold its tiles (one block per SM) and the tile borders
    // (3 sets x 3 planes x 160 floats per tile) fit in dA
    {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // the attribute is per device: set it the first time each device launches here
        static std::mutex attr_mu;
        static bool attr_set[64] = {};
        if (dev >= 0 && dev < 64) {
            std::lock_guard<std::mutex> lock(attr_mu);
            if (!attr_set[dev]) {
                cudaFuncSetAttribute(k_cg_resident, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(kResMaxTiles * kResTileBytes));
                attr_set[dev] = true;
            }
        }
        const int per = (ntiles + sms - 1) / std::max(sms, 1);
        const size_t smem = (size_t)per * kResTileBytes;
        if (per <= kResMaxTiles && (size_t)9 * kResBorder * ntiles <= 3 * N &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_resident, kResThreads, smem) == cudaSuccess &&
            per_sm >= 1) {
            const int blocks = (ntiles + per - 1) / per;
            void *args[] = {&W, &H, (void *)&gx, (void *)&gy, &U, (void *)&U0, &dA, &partA, &partB, &gb,
                            &max_iter, &gap_tol, &state, &trace, &trace_cap};
            lc.add(1);
            return cudaLaunchCooperativeKernel((const void *)k_cg_resident, dim3(blocks), dim3(kResThreads), args,
                                               smem, st);
        }
    }
    // the TMA form needs row pitches of a multiple of 16 bytes (W % 4 == 0) and the driver's encoder
    CUtensorMap maps[5];
    const bool tma = encode_tensor_map_3d(&maps[0], r, W, H, 3, kBoxX, kBoxY, 3) &&
                     encode_tensor_map_3d(&maps[1], dA, W, H, 3, kBoxX, kBoxY, 3) &&
                     encode_tensor_map_3d(&maps[2], dB, W, H, 3, kBoxX, kBoxY, 3) &&
                     encode_tensor_map_3d(&maps[3], U, W, H, 3, kTileX, kTileY, 3) &&
                     encode_tensor_map_3d(&maps[4], r, W, H, 3, kTileX, kTileY, 3);
    if (!tma) std::memset(maps, 0, sizeof(maps));
    const void *kern = tma ? (const void *)k_cg_persistent<true> : (const void *)k_cg_persistent<false>;
    const size_t smem = tma ? kCgTmaSmem : 0;
    if (tma) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // as many blocks as can be resident, then as few as keep the per-block tile count at its minimum (equal
    // tile counts: no block waits at the grid barrier for a straggler with one tile more)
    const int resident = coop_blocks(kern, 1 << 30, smem);
    const int per_block = (ntiles + resident - 1) / resident;
    const int blocks = std::max(1, (ntiles + per_block - 1) / per_block);
    void *args[] = {&W,     &H,       (void *)&gx, (void *)&gy, &U,       (void *)&U0, &r,        &dA,
                    &dB,    &partA,   &partB,      &gb,         &max_iter, &gap_tol,   &state,    &trace,
                    &trace_cap, &maps[0], &maps[1], &maps[2], &maps[3], &maps[4]};
    lc.add(1);
    return cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(kPersistThreads), args, smem, st);
}

int cg_batch_resident_blocks() { return coop_blocks((const void *)k_cg_batch, 1 << 30); }

cudaError_t launch_cg_batch(const CgProblem *d_probs, const int *d_block_prob, int nprob, int blocks, double *partA,
                            double *partB, int *done, GridBarrier gb, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "cg_batch", st);
    void *args[] = {(void *)&d_probs, (void *)&d_block_prob, &nprob, &partA, &partB, &done, &gb};
    lc.add(1);
    return cudaLaunchCooperativeKernel((const void *)k_cg_batch, dim3(blocks), dim3(kPersistThreads), args, 0, st);
}

void *tensor_map_encoder() {
    static void *encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = fn;
        cudaGetLastError();
    });
    return encode;
}

bool encode_tensor_map_3d(CUtensorMap *map, const float *base, int cols, int rows, int planes, int box_x, int box_y,
                          int box_z) {
    const auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encoder());
    if (!encode || !base || cols <= 0 || rows <= 0 || planes <= 0) return false;
    if (((size_t)cols * sizeof(float)) % 16 != 0 || reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)cols * sizeof(float), (cuuint64_t)cols * rows * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, (cuuint32_t)box_z};
    const cuuint32_t estride[3] = {1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_hole_fill_persistent(int W, int H, const int *holes, const int *count, float *A, float *B,
                                        double *part, GridBarrier gb, int max_iter, double *state, cudaStream_t st,
                                        LaunchCounter &lc) {
    // The hole count is on the device: the three forms are queued, and each returns at once unless the count is
    // in its range (one block up to kSmallHoles, one cluster of kHoleCluster blocks up to kHoleCluster times that
    // where the device can place such a cluster, the grid-wide kernel above).
    int handled = kSmallHoles;
    {
        ProfScope _ps(lc, "hole_fill_small", st);
        int dev = 0;
        cudaGetDevice(&dev);
        // per device: the shared-memory attributes, and whether a cluster of kHoleCluster such blocks fits
        static std::mutex mu;
        static int cluster_ok[64] = {};  // 0 unknown, 1 yes, -1 no
        const int slot = (dev >= 0 && dev < 64) ? dev : 0;
        int use_cluster = 0;
        {
            std::lock_guard<std::mutex> lock(mu);
            if (cluster_ok[slot] == 0) {
                cudaError_t e = cudaFuncSetAttribute(k_hole_fill_small<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)kSmallHoleSmem);
                if (e != cudaSuccess) return e;
                int ok = -1;
                if (cudaFuncSetAttribute(k_hole_fill_small<kHoleCluster>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmallHoleSmem) == cudaSuccess) {
                    cudaLaunchConfig_t q = {};
                    cudaLaunchAttribute at[1];
                    at[0].id = cudaLaunchAttributeClusterDimension;
                    at[0].val.clusterDim.x = kHoleCluster;
                    at[0].val.clusterDim.y = 1;
                    at[0].val.clusterDim.z = 1;
                    q.gridDim = dim3(kHoleCluster);
                    q.blockDim = dim3(kSmallThreads);
                    q.dynamicSmemBytes = kSmallHoleSmem;
                    q.attrs = at;
                    q.numAttrs = 1;
                    int nclusters = 0;
                    if (cudaOccupancyMaxActiveClusters(&nclusters, (const void *)k_hole_fill_small<kHoleCluster>, &q) ==
                            cudaSuccess &&
                        nclusters >= 1)
                        ok = 1;
                }
                cudaGetLastError();  // a refused query leaves no error behind
                cluster_ok[slot] = ok;
            }
            use_cluster = cluster_ok[slot] > 0;
        }
        k_hole_fill_small<1><<<1, kSmallThreads, kSmallHoleSmem, st>>>(W, H, holes, count, A, max_iter, state);
        lc.add(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (use_cluster) {
            cudaLaunchConfig_t q = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = kHoleCluster;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            q.gridDim = dim3(kHoleCluster);
            q.blockDim = dim3(kSmallThreads);
            q.dynamicSmemBytes = kSmallHoleSmem;
            q.stream = st;
            q.attrs = at;
            q.numAttrs = 1;
            e = cudaLaunchKernelEx(&q, k_hole_fill_small<kHoleCluster>, W, H, holes, count, A, max_iter, state);
            if (e != cudaSuccess) return e;
            lc.add(1);
            handled = kHoleCluster * kSmallHoles;
        }
    }
    ProfScope _ps(lc, "hole_fill", st);
    const size_t N = (size_t)W * H;
    const int blocks =
        coop_blocks((const void *)k_hole_fill_persistent, (int)((N + kPersistThreads - 1) / kPersistThreads));
    void *args[] = {&W, &H, (void *)&holes, (void *)&count, &A, &B, &part, &gb, &max_iter, &state, &handled};
    lc.add(1);
    return cudaLaunchCooperativeKernel((const void *)k_hole_fill_persistent, dim3(blocks), dim3(kPersistThreads), args,
                                       0, st);
}

void launch_hole_fill_iter(int W, int H, const int *holes, int nholes, const float *Uin, float *Uout, double *partial,
                           cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "hole_fill_iter", st);
    if (nholes <= 0) return;
    k_hole_iter<<<(nholes + 255) / 256, 256, 0, st>>>(W, H, holes, nholes, Uin, Uout, partial);
    lc.add(1);
}

void launch_cg_init(int W, int H, const float *U, const float *gx, const float *gy, float *r, float *d, bool faithful,
                    double *partial, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "cg_init", st);
    k_cg_init<<<cg_grid(W, H), dim3(kCgBX, kCgBY), 0, st>>>(W, H, U, gx, gy, r, d, faithful ? 1 : 0, partial);
    lc.add(1);
}

void launch_cg_apply(int W, int H, const float *d, float lambda, float *q, double *partial, cudaStream_t st,
                     LaunchCounter &lc) {
    k_cg_apply<<<cg_grid(W, H), dim3(kCgBX, kCgBY), 0, st>>>(W, H, d, lambda, q, partial);
    lc.add(1);
}

void launch_cg_update(int W, int H, const float alpha[3], const float *d, const float *q, float *U, float *r,
                      double *partial, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "cg_update", st);
    k_cg_update<<<cg_grid(W, H), dim3(kCgBX, kCgBY), 0, st>>>(W, H, make_float3(alpha[0], alpha[1], alpha[2]), d, q, U,
                                                             r, partial);
    lc.add(1);
}

void launch_cg_dir(int W, int H, const float beta[3], const float *r, float *d, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "cg_dir", st);
    k_cg_dir<<<cg_grid(W, H), dim3(kCgBX, kCgBY), 0, st>>>(W, H, make_float3(beta[0], beta[1], beta[2]), r, d);
    lc.add(1);
}

void launch_reduce_segments(int count, int nseg, const double *partial, double *out, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "reduce_segments", st);
    k_reduce_segments<<<nseg, 1024, 0, st>>>(count, partial, out);
    lc.add(1);
}

void launch_cg_energy(int W, int H, const float *U, const float *U0, const float *gx, const float *gy, double *partial,
                      cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "cg_energy", st);
    k_cg_energy<<<cg_grid(W, H), dim3(kCgBX, kCgBY), 0, st>>>(W, H, U, U0, gx, gy, partial);
    lc.add(1);
}

}  // namespace lfrv

// ====================================================================== allocation-free CG entry point
// lfrv_cg_solve_static runs k_cg_persistent with all of its scratch in one file-scope device array instead of
// context buffers: r and the two direction buffers (3 planes of kStaticPixels floats each), the FP64 block
// partials of phases A and B (4 doubles per block each), 16 doubles of solver state, 64 bytes of barrier words.
namespace {

constexpr size_t kStaticPixels = LFRV_CG_STATIC_MAX_PIXELS;
constexpr int kStaticBlocks = 1024;  // cooperative blocks the partial slots hold (2 per SM for <= 512 SMs)
constexpr size_t kStaticVecBytes = 9 * kStaticPixels * sizeof(float);
constexpr size_t kStaticPartBytes = 2 * 4 * (size_t)kStaticBlocks * sizeof(double);
constexpr size_t kStaticStateBytes = 16 * sizeof(double);
constexpr size_t kStaticBarrierBytes = 64;
constexpr size_t kStaticBytes = kStaticVecBytes + kStaticPartBytes + kStaticStateBytes + kStaticBarrierBytes;
static_assert(kStaticVecBytes % 256 == 0 && kStaticPartBytes % 64 == 0, "scratch sections stay aligned");
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_cg_scratch[kStaticBytes];

std::mutex g_scratch_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};
void *g_scratch_ctx[kMaxDevices] = {};  // the driver context the cached address belongs to

// The calling thread's current driver context (cuCtxGetCurrent through the runtime's entry-point query, so the
// library does not link the driver library directly); nullptr when it cannot be asked.
void *current_driver_context() {
    using Fn = int (*)(void **);
    static Fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<Fn>(f);
        cudaGetLastError();
    });
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

// Address of this device's copy of g_cg_scratch, looked up with that device current the first time a driver
// context of the device calls here. Keyed by the context: after a cudaDeviceReset, or under another context of the
// same ordinal, the module is loaded again and the array moves, so the address is looked up again.
unsigned char *static_scratch(int dev) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    void *ctx = current_driver_context();
    if (!g_scratch_addr[dev] || !ctx || ctx != g_scratch_ctx[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_cg_scratch);
        if (e != cudaSuccess || !p)
            lfrv::raise(LFRV_E_CUDA, "cudaGetSymbolAddress(g_cg_scratch): %s", cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
        g_scratch_ctx[dev] = current_driver_context();  // the runtime has made the primary context current by now
    }
    return g_scratch_addr[dev];
}

}  // namespace

extern "C" int lfrv_cg_solve_static(void *stream, int W, int H, int max_iter, double gap_tol, const float *gx,
                                    const float *gy, float *U, int *iterations, double *gap) {
    using namespace lfrv;
    LFRV_API_BEGIN
    if (W < 2 || H < 2 || !gx || !gy || !U || max_iter < 0) return fail(LFRV_E_ARG, "bad arguments");
    if ((size_t)W * H > kStaticPixels)
        return fail(LFRV_E_ARG, "%d x %d pixels exceed LFRV_CG_STATIC_MAX_PIXELS (%zu)", W, H, kStaticPixels);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(LFRV_E_NODEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(LFRV_E_ARG, "device %d out of range", dev);
    if (persistent_partials() > kStaticBlocks)
        return fail(LFRV_E_ARG, "this device needs more than %d cooperative blocks", kStaticBlocks);
    unsigned char *base = static_scratch(dev);
    float *r = reinterpret_cast<float *>(base);
    float *dA = r + 3 * kStaticPixels, *dB = dA + 3 * kStaticPixels;
    double *partA = reinterpret_cast<double *>(base + kStaticVecBytes), *partB = partA + 4 * kStaticBlocks;
    double *state = partB + 4 * kStaticBlocks;
    unsigned int *bar = reinterpret_cast<unsigned int *>(state + 16);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemsetAsync(bar, 0, kStaticBarrierBytes, st);  // arrival count and error flag start at zero
    if (e != cudaSuccess) return fail(LFRV_E_CUDA, "clearing the barrier words: %s", cudaGetErrorString(e));
    GridBarrier gb;
    gb.count = bar;
    gb.err = reinterpret_cast<int *>(bar + 4);
    LaunchCounter lc;
    e = launch_cg_persistent(W, H, gx, gy, U, r, dA, dB, partA, partB, gb, max_iter, gap_tol, state, st, lc);
    if (e != cudaSuccess) return fail(LFRV_E_CUDA, "k_cg_persistent launch: %s", cudaGetErrorString(e));
    if (iterations || gap) {
        double hs[16];
        int hb[8];
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaMemcpy(hs, state, sizeof(hs), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(hb, bar, sizeof(hb), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(LFRV_E_CUDA, "reading the solver state: %s", cudaGetErrorString(e));
        if (hb[4] != 0) return fail(LFRV_E_TIMEOUT, "a device-side grid barrier gave up waiting");
        if (iterations) *iterations = (int)hs[5];
        if (gap) *gap = hs[4];
    }
    LFRV_API_END
}
