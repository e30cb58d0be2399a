// kernels_learn.cu -- the learned warm start on the 5th-generation tensor cores (sm_103a).
//
// Every convolution of the encoder-decoder, forward and backward, is an implicit GEMM on tcgen05: BF16 operands
// staged in shared memory, FP32 accumulation in tensor memory (TMEM), one thread issuing tcgen05.mma for the CTA,
// completion signalled by tcgen05.commit on an mbarrier, and an epilogue that reads the accumulator with
// tcgen05.ld and applies bias / skip addend / ReLU / ReLU-derivative mask before writing FP32 or BF16.
//
//   forward  : Y[pixel][co]  = sum_(tap,ci) X[pixel * s + tap][ci] W[co][tap,ci]            (k_conv_tc)
//   data grad: dX[pixel][ci] = sum_(tap,co) dY[(pixel - tap) / s][co] W[co][tap,ci]         (k_conv_tc, dgrad)
//   weight   : dW[co][tap,ci] = sum_pixel X[pixel * s + tap][ci] dY[pixel][co]            (k_wgrad_tc, split-K)
//
// Activations are NHWC BF16 (channels contiguous, a multiple of 8), so one 16-byte load of the gather moves 8
// consecutive K elements of one tap. Shared-memory operand layout (K-major, no swizzle): 8 x 16-byte "core
// matrices" (8 rows x 8 bf16). Element (row r, k) of a 64-wide K stage sits at byte
// ((r / 8) * 8 + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2: core matrices adjacent in K are 128 B apart (leading
// byte offset), 8-row groups 1 KB apart (stride byte offset); one MMA (K = 16) reads two core matrices along K, so
// the descriptor start advances 256 B per MMA.
#include <algorithm>
#include <atomic>

#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "device_common.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace lfrv {

namespace {

constexpr int kBM = 128, kBK = 64, kThreads = 128, kStages = 4, kWgStages = 2;

// Shared-memory matrix descriptor: start >> 4 in bits 0-13, leading byte offset >> 4 in 16-29, stride byte
// offset >> 4 in 32-45, the fixed version field (1) in 46-47, base offset 0, layout type 0 (no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo = 128, uint32_t sbo = 1024) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9 = 1, 10-12 = 1), both
// K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc) {
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// Arrives on the mbarrier once every tcgen05.mma this thread issued before it has completed.
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, int cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t tmem, int cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
}

// 16 consecutive accumulator columns of this thread's TMEM lane (warp w of the CTA reads lanes 32 w .. 32 w + 31).
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 16-byte global -> shared copy; bytes = 0 writes zeros (the source is not read).
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Byte offset of the 16-byte chunk (row r, K chunk kc) of a 64-wide stage in the core-matrix layout.
__device__ __forceinline__ uint32_t tile_off(int r, int kc) {
    return (uint32_t)(((r >> 3) * 8 + kc) << 7) + (uint32_t)((r & 7) << 4);
}

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
    return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

__device__ __forceinline__ void unpack8(const uint4 &u, float f[8]) {
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float f[8]) {
    uint4 u;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    return u;
}

// Source pixel of tap (ky, kx) for GEMM row (y, x): forward rows are output pixels (input = y * s - 1 + ky for
// 3 x 3 with padding 1); data-gradient rows are the forward input pixels, whose contributions come from the output
// pixel (y + 1 - ky) / s when that division is exact.
__device__ __forceinline__ bool conv_src(const ConvGemm &g, int y, int x, int ky, int kx, int &iy, int &ix) {
    if (!g.dgrad) {
        iy = y * g.stride + (g.ks == 3 ? ky - 1 : 0);
        ix = x * g.stride + (g.ks == 3 ? kx - 1 : 0);
    } else {
        const int ty = y + (g.ks == 3 ? 1 - ky : 0), tx = x + (g.ks == 3 ? 1 - kx : 0);
        if (ty < 0 || tx < 0) return false;
        if (g.stride == 2) {
            if ((ty | tx) & 1) return false;
            iy = ty >> 1;
            ix = tx >> 1;
        } else {
            iy = ty;
            ix = tx;
        }
    }
    return iy >= 0 && iy < g.Hs && ix >= 0 && ix < g.Ws;
}

// Epilogue of 16 accumulator columns (col .. col + 15) of GEMM row `row` (an output pixel, row-major over batch,
// Ho, Wo): + bias, + add, ReLU, zero where mask <= 0, then the FP32 and / or BF16 stores. With upskip the row's
// value goes, as relu(v + skip), to its 2 x 2 block of the doubled-resolution BF16 output.
__device__ __forceinline__ void conv_store16(const ConvGemm &g, size_t row, int col, float v[16]) {
    const size_t o = row * g.N + col;
    if (g.bias) {
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] += __ldg(g.bias + col + k);
    }
    if (g.add) {
        const uint4 *ap = reinterpret_cast<const uint4 *>(static_cast<const __nv_bfloat16 *>(g.add) + o);
        float tt[8];
        unpack8(ap[0], tt);
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] += tt[k];
        unpack8(ap[1], tt);
#pragma unroll
        for (int k = 0; k < 8; ++k) v[8 + k] += tt[k];
    }
    if (g.upskip) {
        const size_t HW = (size_t)g.Ho * g.Wo;
        const size_t b = row / HW, rem = row - b * HW;
        const int y = (int)(rem / g.Wo), x = (int)(rem - (size_t)y * g.Wo);
        const __nv_bfloat16 *sk = static_cast<const __nv_bfloat16 *>(g.upskip);
        __nv_bfloat16 *out = static_cast<__nv_bfloat16 *>(g.outb);
        size_t oo[4];
        uint4 sv[8];
        // all eight skip loads in flight before the first store
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const size_t hr = (b * 2 * g.Ho + 2 * y + (d >> 1)) * (size_t)(2 * g.Wo) + 2 * x + (d & 1);
            oo[d] = hr * g.N + col;
            const uint4 *sp = reinterpret_cast<const uint4 *>(sk + oo[d]);
            sv[2 * d] = __ldg(sp);
            sv[2 * d + 1] = __ldg(sp + 1);
        }
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            float a[8], c[8], w0[8], w1[8];
            unpack8(sv[2 * d], a);
            unpack8(sv[2 * d + 1], c);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                w0[k] = fmaxf(v[k] + a[k], 0.f);
                w1[k] = fmaxf(v[8 + k] + c[k], 0.f);
            }
            uint4 *bp = reinterpret_cast<uint4 *>(out + oo[d]);
            bp[0] = pack8(w0);
            bp[1] = pack8(w1);
        }
        return;
    }
    if (g.relu) {
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = fmaxf(v[k], 0.f);
    }
    if (g.mask) {
        const uint4 *mp = reinterpret_cast<const uint4 *>(static_cast<const __nv_bfloat16 *>(g.mask) + o);
        float tt[8];
        unpack8(mp[0], tt);
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = tt[k] > 0.f ? v[k] : 0.f;
        unpack8(mp[1], tt);
#pragma unroll
        for (int k = 0; k < 8; ++k) v[8 + k] = tt[k] > 0.f ? v[8 + k] : 0.f;
    }
    if (g.outf) {
        float4 *fp = reinterpret_cast<float4 *>(g.outf + o);
#pragma unroll
        for (int k = 0; k < 4; ++k) fp[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    }
    if (g.outb) {
        uint4 *bp = reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(g.outb) + o);
        bp[0] = pack8(v);
        bp[1] = pack8(v + 8);
    }
}

}  // namespace

// One CTA: 128 GEMM rows (pixels) x BN output channels (columns n0 = blockIdx.y * BN ..), K in 64-wide stages through a kStages-deep
// cp.async ring. Thread 0 issues the four K = 16 MMAs of a stage once the stage has landed and commits them to
// the stage's mbarrier; a slot is refilled only after the mbarrier shows that the MMAs reading it completed.
template <int BN>
__global__ void __launch_bounds__(kThreads) k_conv_tc(const ConvGemm g, int *err) {
    extern __shared__ uint8_t dsm[];
    constexpr int kAB = kBM * kBK * 2, kStage = kAB + BN * kBK * 2;
    constexpr int kCols = BN < 32 ? 32 : BN;
    __shared__ __align__(8) uint64_t bars[kStages];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    uint8_t *base = align1024(dsm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int M = g.batch * g.Ho * g.Wo, HWo = g.Ho * g.Wo;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    if (warp == 0) tmem_alloc(&tmem_slot, kCols);
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        s_fail = 0;
        fence_proxy_async_smem();
    }
    // this thread's eight gather rows (fixed over K) and K chunk
    const int rlo = tid & 7, kc = (tid >> 3) & 7, rhi = tid >> 6;
    int rbase[8], ry[8], rx[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int m = m0 + (rhi + 2 * j) * 8 + rlo;
        if (m < M) {
            const int b = m / HWo, rem = m - b * HWo, y = rem / g.Wo;
            rbase[j] = b * g.Hs * g.Ws;
            ry[j] = y;
            rx[j] = rem - y * g.Wo;
        } else {
            rbase[j] = 0;
            ry[j] = -(1 << 28);
            rx[j] = -(1 << 28);
        }
    }
    const __nv_bfloat16 *src = static_cast<const __nv_bfloat16 *>(g.src);
    const __nv_bfloat16 *wt = static_cast<const __nv_bfloat16 *>(g.wt);
    const uint32_t sbase = smem_u32(base);
    auto load_stage = [&](int kt, int slot) {
        const uint32_t sa = sbase + slot * kStage, sb = sa + kAB;
        const int k = kt * kBK + kc * 8;
        const bool kvalid = k < g.K;
        int tap = 0, ci = 0;
        if (kvalid) {
            tap = k / g.C;
            ci = k - tap * g.C;
        }
        const int ky = (g.ks == 3) ? tap / 3 : 0, kx = (g.ks == 3) ? tap - ky * 3 : 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int iy = 0, ix = 0;
            const bool ok = kvalid && conv_src(g, ry[j], rx[j], ky, kx, iy, ix);
            const __nv_bfloat16 *p = ok ? src + (size_t)(rbase[j] + iy * g.Ws + ix) * g.C + ci : src;
            cp_async16(sa + tile_off((rhi + 2 * j) * 8 + rlo, kc), p, ok ? 16 : 0);
        }
#pragma unroll
        for (int j = 0; j < BN / 16; ++j) {
            const int r = (rhi + 2 * j) * 8 + rlo;
            cp_async16(sb + tile_off(r, kc), wt + (size_t)(n0 + r) * g.ldw + kt * kBK + kc * 8, 16);
        }
    };
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = idesc_bf16_f32(kBM, BN);
    const int nk = (g.K + kBK - 1) / kBK;
#pragma unroll 1
    for (int s = 0; s < kStages - 1; ++s) {
        if (s < nk) load_stage(s, s);
        cp_async_commit();
    }
    int issued = 0;  // stages whose MMAs were committed
#pragma unroll 1
    for (int kt = 0; kt < nk; ++kt) {
        const int slot = kt % kStages;
        cp_async_wait<kStages - 2>();  // stage kt has landed
        fence_proxy_async_smem();      // make this thread's shared-memory writes visible to the tensor core
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (s_fail) break;
        if (tid == 0) {
            const uint32_t a = sbase + slot * kStage, b = a + kAB;
#pragma unroll
            for (int s = 0; s < kBK / 16; ++s)
                tc_mma(tmem, smem_desc(a + s * 256), smem_desc(b + s * 256), idesc, (kt > 0 || s > 0) ? 1 : 0);
            tc_commit(&bars[slot]);
        }
        issued = kt + 1;
        const int nxt = kt + kStages - 1;
        if (nxt < nk) {
            bool ok = true;
            if (kt >= 1) ok = mbar_wait(&bars[(kt - 1) % kStages], ((kt - 1) / kStages) & 1, kSpinLimit);
            if (ok) load_stage(nxt, nxt % kStages);
            else {
                s_fail = 1;
                atomicExch(err, 1);
            }
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    // the last commit covers every MMA issued before it
    bool done = true;
    if (issued > 0) done = mbar_wait(&bars[(issued - 1) % kStages], ((issued - 1) / kStages) & 1, kSpinLimit);
    if (!done) {
        s_fail = 1;
        atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!s_fail && issued == nk) {
        const int m = m0 + warp * 32 + lane;
        const bool row_ok = m < M;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (!row_ok) continue;
            conv_store16(g, (size_t)m, n0 + c0, v);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, kCols);
}

// Stride-1 3 x 3 convolution (or its data gradient, taps mirrored) with the input tile resident in shared memory.
// A CTA computes R output rows x 128 columns (x0 .. x0 + 127) x BN channels: it loads the (R + 2) x 130 input pixels
// around them once, in a layout where consecutive pixels are consecutive 16-byte rows of the core matrices
// (stride byte offset 128) and the 8-channel chunks are kLboA apart (leading byte offset), so the A operand of
// tap (ky, kx) for output row i is the same tile read from pixel (i + ky) * 130 + kx on: nine shifted descriptors
// instead of nine gathers. The weights stream per tap through a 3-slot cp.async ring. TMEM: R accumulators of BN
// columns. Needs W % 128 == 0, H % R == 0, C % 16 == 0.
constexpr int kTileW = 130, kTapStages = 3;

__host__ __device__ constexpr int tile_lbo_px(int R) { return ((R + 2) * kTileW) | 1; }  // odd: spreads the banks

template <int BN, int R>
__global__ void __launch_bounds__(kThreads) k_conv_tile_tc(const ConvGemm g, int *err) {
    extern __shared__ uint8_t dsm[];
    constexpr int kCols = (R * BN) < 32 ? 32 : (R * BN);
    constexpr int npix = (R + 2) * kTileW, lbo_px = tile_lbo_px(R);
    __shared__ __align__(8) uint64_t bars[kTapStages];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    uint8_t *base = align1024(dsm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int C = g.C, chunks = C >> 3;
    const int strips = g.Wo >> 7, yblocks = g.Ho / R;
    int blk = blockIdx.x;
    const int strip = blk % strips;
    blk /= strips;
    const int yb = blk % yblocks, b = blk / yblocks;
    const int x0 = strip << 7, y0 = yb * R, n0 = blockIdx.y * BN;
    const uint32_t lboA = (uint32_t)lbo_px * 16u;
    const uint32_t sA = smem_u32(base), sB = sA + (uint32_t)chunks * lboA;
    const uint32_t bstage = (uint32_t)BN * (uint32_t)C * 2u;  // bytes of one tap's weights
    if (warp == 0) tmem_alloc(&tmem_slot, kCols);
    if (tid == 0) {
        for (int s = 0; s < kTapStages; ++s) mbar_init(&bars[s], 1);
        s_fail = 0;
        fence_proxy_async_smem();
    }
    const __nv_bfloat16 *src = static_cast<const __nv_bfloat16 *>(g.src);
    const __nv_bfloat16 *wt = static_cast<const __nv_bfloat16 *>(g.wt);
    // the input tile (zero outside the image): thread q -> pixel q / chunks, chunk q % chunks (coalesced reads)
    const size_t img = (size_t)b * g.Hs * g.Ws;
    for (int q = tid; q < npix * chunks; q += kThreads) {
        const int p = q / chunks, j = q - p * chunks;
        const int rr = p / kTileW, cc = p - rr * kTileW;
        const int iy = y0 - 1 + rr, ix = x0 - 1 + cc;
        const bool ok = iy >= 0 && iy < g.Hs && ix >= 0 && ix < g.Ws;
        const __nv_bfloat16 *gp = ok ? src + (img + (size_t)iy * g.Ws + ix) * C + j * 8 : src;
        cp_async16(sA + (uint32_t)j * lboA + (uint32_t)p * 16u, gp, ok ? 16 : 0);
    }
    cp_async_commit();
    // one tap's weights: B[n][c] = wt[n0 + n][tap * C + c], chunk-major (chunk j at j * BN * 16, row n at n * 16)
    auto load_tap = [&](int t, int slot) {
        const uint32_t dst = sB + (uint32_t)slot * bstage;
        for (int q = tid; q < BN * chunks; q += kThreads) {
            const int n = q % BN, j = q / BN;
            cp_async16(dst + (uint32_t)(j * BN + n) * 16u, wt + (size_t)(n0 + n) * g.ldw + t * C + j * 8, 16);
        }
    };
    load_tap(0, 0);
    cp_async_commit();
    load_tap(1, 1);
    cp_async_commit();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = idesc_bf16_f32(kBM, BN);
    int issued = 0;
#pragma unroll 1
    for (int t = 0; t < 9; ++t) {
        cp_async_wait<1>();  // the tile and this tap's weights have landed
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (s_fail) break;
        if (tid == 0) {
            const int ky = t / 3, kx = t - 3 * (t / 3);
            const int sy = g.dgrad ? 2 - ky : ky, sx = g.dgrad ? 2 - kx : kx;
            const uint32_t bb = sB + (uint32_t)(t % kTapStages) * bstage;
            for (int i = 0; i < R; ++i) {
                const uint32_t a0 = sA + (uint32_t)((i + sy) * kTileW + sx) * 16u;
                for (int s = 0; s < C / 16; ++s)
                    tc_mma(tmem + (uint32_t)(i * BN), smem_desc(a0 + (uint32_t)(2 * s) * lboA, lboA, 128),
                           smem_desc(bb + (uint32_t)(2 * s) * (uint32_t)BN * 16u, (uint32_t)BN * 16u, 128), idesc,
                           (t > 0 || s > 0) ? 1 : 0);
            }
            tc_commit(&bars[t % kTapStages]);
        }
        issued = t + 1;
        if (t + 2 < 9) {
            bool ok = true;
            if (t >= 1) ok = mbar_wait(&bars[(t - 1) % kTapStages], ((t - 1) / kTapStages) & 1, kSpinLimit);
            if (ok) load_tap(t + 2, (t + 2) % kTapStages);
            else {
                s_fail = 1;
                atomicExch(err, 1);
            }
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    bool done = true;
    if (issued > 0) done = mbar_wait(&bars[(issued - 1) % kTapStages], ((issued - 1) / kTapStages) & 1, kSpinLimit);
    if (!done) {
        s_fail = 1;
        atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!s_fail && issued == 9) {
        const int m = warp * 32 + lane;
#pragma unroll 1
        for (int i = 0; i < R; ++i) {
            const size_t row = ((size_t)b * g.Ho + y0 + i) * g.Wo + x0 + m;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 16) {
                float v[16];
                tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(i * BN + c0), v);
                conv_store16(g, row, n0 + c0, v);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, kCols);
}

// TMA-fed convolution with warp-specialised roles. A CTA owns a patch of bh x bw = 128 output pixels of one image
// (one row of 128, or 128 / Wo whole rows) and BN output channels. The K loop runs over (tap, 64-channel block):
// per stage, one thread issues a strided 4-D TMA box of the activations (64 channels x the patch's input pixels,
// element stride = the convolution stride; padding and channels past C arrive as zeros) and a 2-D box of the
// weights, both 128-byte swizzled, onto a full mbarrier with the stage's byte count. A second thread waits for the
// stage, issues its four K = 16 MMAs and commits them to the stage's empty mbarrier, which releases the slot to the
// producer. After the last stage the MMA thread commits to `done`, and the four warps read the accumulator.
// Forward convolutions of stride 1 or 2 (3 x 3 or 1 x 1) and the data gradient of stride-1 layers (taps mirrored).
constexpr int kTmaStages = 4;

// K-major operand in the 128-byte swizzle: 128-byte rows (64 bf16), 8-row atoms of 1 KB (stride byte offset),
// layout type 2 in bits 61-63; successive K = 16 slices start 32 B apart inside the atom.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

template <int BN>
__global__ void __launch_bounds__(kThreads) k_conv_tma(const ConvGemm g, const __grid_constant__ CUtensorMap mapA,
                                                       const __grid_constant__ CUtensorMap mapB, int bw, int bh,
                                                       int cblocks, int *err) {
    extern __shared__ uint8_t dsm[];
    constexpr int kA = kBM * 128, kStage = kA + BN * 128;
    constexpr int kCols = BN < 32 ? 32 : BN;
    __shared__ __align__(8) uint64_t full[kTmaStages], empty[kTmaStages], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    uint8_t *base = align1024(dsm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int pxn = g.Wo / bw, pyn = g.Ho / bh;
    int blk = blockIdx.x;
    const int pxi = blk % pxn;
    blk /= pxn;
    const int pyi = blk % pyn, b = blk / pyn;
    const int ox0 = pxi * bw, oy0 = pyi * bh, n0 = blockIdx.y * BN;
    const int nk = g.ks * g.ks * cblocks;
    if (warp == 0) tmem_alloc(&tmem_slot, kCols);
    if (tid == 0) {
        for (int s = 0; s < kTmaStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        s_fail = 0;
        fence_proxy_async_smem();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (warp == 0 && lane == 0) {
        // producer
        for (int kt = 0; kt < nk; ++kt) {
            const int slot = kt % kTmaStages, use = kt / kTmaStages;
            if (kt >= kTmaStages && !mbar_wait(&empty[slot], (use - 1) & 1, kSpinLimit)) {
                s_fail = 1;
                atomicExch(err, 1);
                break;
            }
            const int tap = kt / cblocks, cb = kt - tap * cblocks;
            int sx = ox0 * g.stride, sy = oy0 * g.stride;
            if (g.ks == 3) {
                const int ky = tap / 3, kx = tap - 3 * (tap / 3);
                if (!g.dgrad) {
                    sx += kx - 1;
                    sy += ky - 1;
                } else {
                    sx = ox0 + 1 - kx;
                    sy = oy0 + 1 - ky;
                }
            }
            uint8_t *sa = base + slot * kStage;
            mbar_arrive_expect_tx(&full[slot], (unsigned)kStage);
            tma_load_4d(sa, &mapA, cb * 64, sx, sy, b, &full[slot]);
            tma_load_2d(sa + kA, &mapB, tap * g.C + cb * 64, n0, &full[slot]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = idesc_bf16_f32(kBM, BN);
        for (int kt = 0; kt < nk; ++kt) {
            const int slot = kt % kTmaStages, use = kt / kTmaStages;
            if (!mbar_wait(&full[slot], use & 1, kSpinLimit)) {
                s_fail = 1;
                atomicExch(err, 1);
                break;
            }
            tc_fence_after();
            const uint32_t a = smem_u32(base + slot * kStage), bb = a + kA;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                tc_mma(tmem, smem_desc_sw128(a + 32 * k), smem_desc_sw128(bb + 32 * k), idesc, (kt > 0 || k > 0) ? 1 : 0);
            tc_commit(&empty[slot]);
        }
        tc_commit(&done);  // arrives once every MMA issued above has completed
    }
    __syncthreads();
    if (!mbar_wait(&done, 0, kSpinLimit)) {
        s_fail = 1;
        atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!s_fail) {
        const int m = warp * 32 + lane;
        const int oy = oy0 + m / bw, ox = ox0 + m % bw;
        const size_t row = ((size_t)b * g.Ho + oy) * g.Wo + ox;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            conv_store16(g, row, n0 + c0, v);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, kCols);
}

// Weight gradient: GEMM rows are the (tap, ci) rows of dW^T (padded to 128), N = the stored output channels, the
// reduction runs over the output pixels of this split. Both operands are pixel-major in global memory, so each
// 16-byte load (8 channels of one pixel) is written transposed into a column of a core matrix. Double-buffered:
// the global loads of stage k overlap the MMAs of stage k - 1. Result: FP32 partial[split][row][co].
template <int BN>
__global__ void __launch_bounds__(kThreads) k_wgrad_tc(const WgradGemm g, int *err) {
    extern __shared__ uint8_t dsm[];
    constexpr int kAB = kBM * kBK * 2, kStage = kAB + BN * kBK * 2;
    constexpr int kCols = BN < 32 ? 32 : BN;
    constexpr int kBChunks = BN / 16;  // per thread
    __shared__ __align__(8) uint64_t bars[kWgStages];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    uint8_t *base = align1024(dsm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int HWo = g.Ho * g.Wo, P = g.batch * HWo;
    const int m0 = blockIdx.x * kBM;
    const int p0 = blockIdx.y * g.chunk, p1 = min(P, p0 + g.chunk);
    if (warp == 0) tmem_alloc(&tmem_slot, kCols);
    if (tid == 0) {
        for (int s = 0; s < kWgStages; ++s) mbar_init(&bars[s], 1);
        s_fail = 0;
        fence_proxy_async_smem();
    }
    const int pk = tid & 63, grp = tid >> 6;  // this thread's pixel column and first 8-row group
    // rows of the A chunks: group G = grp + 2 j holds rows m0 + 8 G .. + 7 = 8 channels of one tap
    int atap[8], aci[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int r0 = m0 + (grp + 2 * j) * 8;
        if (r0 < g.Kf) {
            atap[j] = r0 / g.Cin;
            aci[j] = r0 - atap[j] * g.Cin;
        } else {
            atap[j] = -1;
            aci[j] = 0;
        }
    }
    const __nv_bfloat16 *X = static_cast<const __nv_bfloat16 *>(g.x);
    const __nv_bfloat16 *DY = static_cast<const __nv_bfloat16 *>(g.dy);
    const uint32_t sbase = smem_u32(base);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = idesc_bf16_f32(kBM, BN);
    const int nk = (p1 - p0 + kBK - 1) / kBK;
    int issued = 0;
#pragma unroll 1
    for (int kt = 0; kt < nk; ++kt) {
        const int slot = kt % kWgStages;
        // global loads of this stage (registers)
        const int p = p0 + kt * kBK + pk;
        const bool pv = p < p1;
        int b = 0, oy = 0, ox = 0;
        if (pv) {
            b = p / HWo;
            const int rem = p - b * HWo;
            oy = rem / g.Wo;
            ox = rem - oy * g.Wo;
        }
        uint4 va[8], vb[kBChunks];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            va[j] = make_uint4(0, 0, 0, 0);
            if (pv && atap[j] >= 0) {
                int iy = oy * g.stride, ix = ox * g.stride;
                if (g.ks == 3) {
                    const int ky = atap[j] / 3;
                    iy += ky - 1;
                    ix += atap[j] - ky * 3 - 1;
                }
                if (iy >= 0 && iy < g.Hx && ix >= 0 && ix < g.Wx)
                    va[j] = __ldg(reinterpret_cast<const uint4 *>(X + ((size_t)b * g.Hx * g.Wx + (size_t)iy * g.Wx + ix) * g.Cin + aci[j]));
            }
        }
#pragma unroll
        for (int j = 0; j < kBChunks; ++j) {
            vb[j] = make_uint4(0, 0, 0, 0);
            if (pv) vb[j] = __ldg(reinterpret_cast<const uint4 *>(DY + (size_t)p * g.Cout + (grp + 2 * j) * 8));
        }
        // the slot was last read by the MMAs of stage kt - 2
        if (kt >= kWgStages) {
            if (!mbar_wait(&bars[slot], ((kt - kWgStages) / kWgStages) & 1, kSpinLimit)) {
                s_fail = 1;
                atomicExch(err, 1);
            }
        }
        tc_fence_before();
        __syncthreads();
        if (s_fail) break;
        uint8_t *sa = base + slot * kStage, *sb = sa + kAB;
        const int colb = ((pk >> 3) << 7) + ((pk & 7) << 1);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint16_t *h = reinterpret_cast<const uint16_t *>(&va[j]);
            uint8_t *dst = sa + ((grp + 2 * j) << 10) + colb;
#pragma unroll
            for (int i = 0; i < 8; ++i) *reinterpret_cast<uint16_t *>(dst + (i << 4)) = h[i];
        }
#pragma unroll
        for (int j = 0; j < kBChunks; ++j) {
            const uint16_t *h = reinterpret_cast<const uint16_t *>(&vb[j]);
            uint8_t *dst = sb + ((grp + 2 * j) << 10) + colb;
#pragma unroll
            for (int i = 0; i < 8; ++i) *reinterpret_cast<uint16_t *>(dst + (i << 4)) = h[i];
        }
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a = sbase + slot * kStage, bb = a + kAB;
#pragma unroll
            for (int s = 0; s < kBK / 16; ++s)
                tc_mma(tmem, smem_desc(a + s * 256), smem_desc(bb + s * 256), idesc, (kt > 0 || s > 0) ? 1 : 0);
            tc_commit(&bars[slot]);
        }
        issued = kt + 1;
    }
    bool done = true;
    if (issued > 0) done = mbar_wait(&bars[(issued - 1) % kWgStages], ((issued - 1) / kWgStages) & 1, kSpinLimit);
    if (!done) {
        s_fail = 1;
        atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (!s_fail) {
        const int r = warp * 32 + lane;
        float *out = g.partial + ((size_t)blockIdx.y * g.Mpad + m0 + r) * BN;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if (issued > 0) tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            else {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            float4 *fp = reinterpret_cast<float4 *>(out + c0);
#pragma unroll
            for (int i = 0; i < 4; ++i) fp[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, kCols);
}

// dW[co][k] = sum over splits of partial[split][k][co] (k < Kf, co < Cout), written into the flat FP32 gradient.
__global__ void k_wgrad_reduce(int splits, int Mpad, int Cst, int Kf, int Cout, const float *__restrict__ partial,
                               float *__restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Kf * Cout) return;
    const int co = i / Kf, k = i - co * Kf;
    float s = 0.f;
    for (int sp = 0; sp < splits; ++sp) s += partial[((size_t)sp * Mpad + k) * Cst + co];
    grad[i] = s;
}

// Column sums of a BF16 [P][C] tensor (bias gradients): per-block partials[block][C] in a fixed order.
__global__ void __launch_bounds__(256) k_colsum(int P, int C, const __nv_bfloat16 *__restrict__ dy,
                                                float *__restrict__ partial) {
    __shared__ float sh[256];
    const int lanes = 256 / C, c = threadIdx.x % C, l = threadIdx.x / C;
    float s = 0.f;
    if (l < lanes)
        for (int p = blockIdx.x * lanes + l; p < P; p += gridDim.x * lanes) s += __bfloat162float(dy[(size_t)p * C + c]);
    sh[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int j = 0; j < lanes; ++j) t += sh[j * C + threadIdx.x];
        partial[(size_t)blockIdx.x * C + threadIdx.x] = t;
    }
}

__global__ void k_colsum_final(int blocks, int C, int Creal, const float *__restrict__ partial, float *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= Creal) return;
    float t = 0.f;
    for (int b = 0; b < blocks; ++b) t += partial[(size_t)b * C + c];
    out[c] = t;
}

// s = relu(up2(t) + skip): t at (Hl, Wl), skip and s at (2 Hl, 2 Wl), C channels (8 per thread).
__global__ void k_upsample_add_relu(int batch, int Hl, int Wl, int C, const __nv_bfloat16 *__restrict__ t,
                                    const __nv_bfloat16 *__restrict__ skip, __nv_bfloat16 *__restrict__ s) {
    const int C8 = C >> 3, W = 2 * Wl, H = 2 * Hl;
    const size_t total = (size_t)batch * H * W * C8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % C8);
        const size_t pix = i / C8;
        const int x = (int)(pix % W);
        const size_t r = pix / W;
        const int y = (int)(r % H), b = (int)(r / H);
        const size_t lo = (((size_t)b * Hl + (y >> 1)) * Wl + (x >> 1)) * C + c8 * 8;
        float a[8], k[8];
        unpack8(*reinterpret_cast<const uint4 *>(t + lo), a);
        unpack8(*reinterpret_cast<const uint4 *>(skip + pix * C + c8 * 8), k);
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fmaxf(a[j] + k[j], 0.f);
        *reinterpret_cast<uint4 *>(s + pix * C + c8 * 8) = pack8(a);
    }
}

// dt = sum of the 2 x 2 block of ds (the adjoint of nearest upsampling).
__global__ void k_down_sum(int batch, int Hl, int Wl, int C, const __nv_bfloat16 *__restrict__ ds,
                           __nv_bfloat16 *__restrict__ dt) {
    const int C8 = C >> 3, W = 2 * Wl;
    const size_t total = (size_t)batch * Hl * Wl * C8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % C8);
        const size_t pix = i / C8;
        const int x = (int)(pix % Wl);
        const size_t r = pix / Wl;
        const int y = (int)(r % Hl), b = (int)(r / Hl);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const size_t hp = ((size_t)b * 2 * Hl + 2 * y + (d >> 1)) * W + 2 * x + (d & 1);
            unpack8(*reinterpret_cast<const uint4 *>(ds + hp * C + c8 * 8), v);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] += v[j];
        }
        *reinterpret_cast<uint4 *>(dt + pix * C + c8 * 8) = pack8(acc);
    }
}

// Output head: pred = u0 + y[:, 0:3] (planar per image), and with a target the loss 1/(3 P) sum (pred - target)^2,
// its gradient dy = 2 (pred - target) / (3 P) as BF16 [P][Cy] (zero in the padding channels), per-block loss
// partials in FP64.
__global__ void __launch_bounds__(256) k_output_head(int batch, int HW, int Cy, const float *__restrict__ y,
                                                     const float *__restrict__ u0, const float *__restrict__ target,
                                                     float *__restrict__ pred, __nv_bfloat16 *__restrict__ dy,
                                                     double *__restrict__ loss_partial) {
    __shared__ double sh[8];
    const size_t P = (size_t)batch * HW;
    const float scale = 2.0f / (3.0f * (float)P);
    double acc = 0.0;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const size_t b = p / HW, o = p - b * HW;
        float d[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const size_t q = (b * 3 + c) * HW + o;
            const float v = u0[q] + y[p * Cy + c];
            if (pred) pred[q] = v;
            d[c] = target ? v - target[q] : 0.f;
            acc += (double)d[c] * d[c];
        }
        if (dy) {
            for (int c = 0; c < Cy; ++c)
                dy[p * Cy + c] = __float2bfloat16_rn(c < 3 ? d[c] * scale : 0.f);
        }
    }
    acc = block_sum<256>(acc, sh);
    if (threadIdx.x == 0 && loss_partial) loss_partial[blockIdx.x] = acc;
}

// Adam on the flat FP32 parameters (bias-corrected step sizes computed on the host).
__global__ void k_adam(size_t n, float *__restrict__ w, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, float lr_t, float b1, float b2, float eps_t) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr_t * mi / (sqrtf(vi) + eps_t);
    }
}

// BF16 GEMM copies of one layer's FP32 weights w[co][tap * Cin + ci]: Wb[co][k] (Cst x Kpad, zero padded) for the
// forward pass and Wt[ci][tap * Cst + co] (Cin x Kdpad) for the data gradient.
__global__ void k_pack_weights(int Cout, int Cst, int Cin, int taps, int Kpad, int Kdpad, const float *__restrict__ w,
                               __nv_bfloat16 *__restrict__ Wb, __nv_bfloat16 *__restrict__ Wt) {
    const int Kf = taps * Cin;
    const size_t nb = (size_t)Cst * Kpad, nt = (size_t)Cin * Kdpad;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nb + nt; i += (size_t)gridDim.x * blockDim.x) {
        if (i < nb) {
            const int co = (int)(i / Kpad), k = (int)(i % Kpad);
            Wb[i] = __float2bfloat16_rn((co < Cout && k < Kf) ? w[(size_t)co * Kf + k] : 0.f);
        } else {
            const size_t j = i - nb;
            const int ci = (int)(j / Kdpad), kd = (int)(j % Kdpad);
            const int tap = kd / Cst, co = kd - tap * Cst;
            float val = 0.f;
            if (tap < taps && co < Cout) val = w[(size_t)co * Kf + tap * Cin + ci];
            Wt[j] = __float2bfloat16_rn(val);
        }
    }
}

// ------------------------------------------------------------------ launchers
template <int BN>
static cudaError_t conv_launch(const ConvGemm &g, int *err, cudaStream_t st) {
    constexpr int smem = kStages * (kBM * kBK * 2 + BN * kBK * 2) + 1024;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_conv_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int M = g.batch * g.Ho * g.Wo;
    k_conv_tc<BN><<<dim3((M + kBM - 1) / kBM, g.N / BN), kThreads, smem, st>>>(g, err);
    return cudaGetLastError();
}

template <int BN, int R>
static cudaError_t tile_launch(const ConvGemm &g, int smem, int *err, cudaStream_t st) {
    static int attr = 0;
    if (smem > attr) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_conv_tile_tc<BN, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = smem;
    }
    const dim3 grid(g.batch * (g.Ho / R) * (g.Wo >> 7), g.N / BN);
    k_conv_tile_tc<BN, R><<<grid, kThreads, smem, st>>>(g, err);
    return cudaGetLastError();
}

// The resident-tile kernel's shape for a stride-1 3 x 3 layer (forward, or data gradient of a stride-1 layer), or
// false when it does not apply (rows not a multiple of 128, channels not a multiple of 16, no shape that fits).
static bool tile_shape(const ConvGemm &g, int &R, int &BN, int &smem) {
    if (g.ks != 3 || g.stride != 1 || g.Wo % 128 || g.C % 16 || g.Hs != g.Ho || g.Ws != g.Wo) return false;
    if (g.ldw < 9 * g.C) return false;
    int best = -1;
    for (int r : {4, 2, 1}) {
        if (g.Ho % r) continue;
        for (int bn = g.N; bn >= 16 && bn >= g.N / 2; bn >>= 1) {
            if (r * bn > 256 || bn > 128) continue;
            const int sm = (g.C / 8) * tile_lbo_px(r) * 16 + kTapStages * bn * g.C * 2 + 1024;
            if (sm > 200 * 1024) continue;
            const int ctas = g.batch * (g.Ho / r) * (g.Wo / 128) * (g.N / bn);
            const int score = std::min(ctas, 2 * 148);
            if (score > best) {
                best = score;
                R = r;
                BN = bn;
                smem = sm;
            }
        }
    }
    return best > 0;
}

static cudaError_t launch_tile(const ConvGemm &g, int R, int BN, int smem, int *err, cudaStream_t st) {
#define LFRV_TILE_CASE(bn, r) \
    if (BN == bn && R == r) return tile_launch<bn, r>(g, smem, err, st);
    LFRV_TILE_CASE(16, 1) LFRV_TILE_CASE(16, 2) LFRV_TILE_CASE(16, 4)
    LFRV_TILE_CASE(32, 1) LFRV_TILE_CASE(32, 2) LFRV_TILE_CASE(32, 4)
    LFRV_TILE_CASE(64, 1) LFRV_TILE_CASE(64, 2) LFRV_TILE_CASE(64, 4)
    LFRV_TILE_CASE(128, 1) LFRV_TILE_CASE(128, 2)
#undef LFRV_TILE_CASE
    return cudaErrorInvalidValue;
}

// Patch of the TMA kernel (bw x bh = 128 output pixels), or false when the layer does not tile that way or is a
// data gradient of stride 2.
static bool tma_shape(const ConvGemm &g, int &bw, int &bh) {
    if (g.ks != 1 && g.ks != 3) return false;
    if (g.dgrad && g.stride != 1) return false;
    if (g.C % 8 || g.C < 8) return false;
    if (g.Wo >= 128) {
        if (g.Wo % 128) return false;
        bw = 128;
        bh = 1;
    } else {
        if (128 % g.Wo) return false;
        bw = g.Wo;
        bh = 128 / g.Wo;
        if (g.Ho % bh) return false;
    }
    const int s = g.dgrad ? 1 : g.stride;
    return bw * s <= 256 && bh * s <= 256;
}

// Activation map: dims (C, W, H, batch) of NHWC BF16, box (64, bw s, bh s, 1) with element strides (1, s, s, 1);
// weight map: dims (ldw, N), box (64, BN). Both with the 128-byte swizzle and zero fill outside the tensor.
static bool encode_conv_maps(const ConvGemm &g, int bw, int bh, int BN, CUtensorMap *mA, CUtensorMap *mB) {
    const auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encoder());
    if (!encode) return false;
    const int s = g.dgrad ? 1 : g.stride;
    const cuuint64_t adims[4] = {(cuuint64_t)g.C, (cuuint64_t)g.Ws, (cuuint64_t)g.Hs, (cuuint64_t)g.batch};
    const cuuint64_t astr[3] = {(cuuint64_t)g.C * 2, (cuuint64_t)g.Ws * g.C * 2, (cuuint64_t)g.Hs * g.Ws * g.C * 2};
    const cuuint32_t abox[4] = {64, (cuuint32_t)(bw * s), (cuuint32_t)(bh * s), 1};
    const cuuint32_t aes[4] = {1, (cuuint32_t)s, (cuuint32_t)s, 1};
    if (encode(mA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(g.src), adims, astr, abox, aes,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const cuuint64_t bdims[2] = {(cuuint64_t)g.ldw, (cuuint64_t)g.N};
    const cuuint64_t bstr[1] = {(cuuint64_t)g.ldw * 2};
    const cuuint32_t bbox[2] = {64, (cuuint32_t)BN};
    const cuuint32_t bes[2] = {1, 1};
    return encode(mB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(g.wt), bdims, bstr, bbox, bes,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
static cudaError_t tma_launch(const ConvGemm &g, int bw, int bh, const CUtensorMap &mA, const CUtensorMap &mB, int *err,
                              cudaStream_t st) {
    constexpr int smem = kTmaStages * (kBM * 128 + BN * 128) + 1024;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_conv_tma<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int cblocks = (g.C + 63) / 64;
    const dim3 grid(g.batch * (g.Ho / bh) * (g.Wo / bw), g.N / BN);
    k_conv_tma<BN><<<grid, kThreads, smem, st>>>(g, mA, mB, bw, bh, cblocks, err);
    return cudaGetLastError();
}

// Which convolution kernel a layer uses: the TMA kernel where its patch tiling applies, else the resident-tile
// kernel (stride-1 3 x 3 on 128-pixel rows), else the cp.async gather. The preference (0 all, 1 no TMA kernel,
// 2 the gather only) restricts the choice; a kernel that does not apply falls through to the next.
static std::atomic<int> g_conv_pref{0};
void set_conv_kernel_pref(int pref) { g_conv_pref.store(pref); }
static int conv_kernel_pref() { return g_conv_pref.load(); }

cudaError_t launch_conv_tc(const ConvGemm &g, int *err, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, g.dgrad ? "conv_dgrad_tc" : "conv_fwd_tc", st);
    if (g.N != 16 && g.N != 32 && g.N != 64 && g.N != 128 && g.N != 256) return cudaErrorInvalidValue;
    const int pref = conv_kernel_pref();
    // the resident-tile kernel reads each input pixel ~1.5 times, the TMA kernel once per tap in 64-channel boxes:
    // with fewer than 64 channels the tile kernel moves fewer bytes
    {
        int R = 0, BN = 0, smem = 0;
        if (pref <= 1 && g.C < 64 && tile_shape(g, R, BN, smem)) {
            const cudaError_t e = launch_tile(g, R, BN, smem, err, st);
            lc.add(1);
            return e;
        }
    }
    {
        int bw = 0, bh = 0;
        CUtensorMap mA, mB;
        int bn = g.N;
        const bool tma = pref == 0 && tma_shape(g, bw, bh);
        if (tma) {
            const int mtiles = g.batch * (g.Ho / bh) * (g.Wo / bw);
            while (bn > 32 && mtiles * (g.N / bn) < 120) bn >>= 1;
        }
        // a map the driver does not accept sends the layer to the other kernels
        if (tma && encode_conv_maps(g, bw, bh, bn, &mA, &mB)) {
            cudaError_t e;
            switch (bn) {
                case 16: e = tma_launch<16>(g, bw, bh, mA, mB, err, st); break;
                case 32: e = tma_launch<32>(g, bw, bh, mA, mB, err, st); break;
                case 64: e = tma_launch<64>(g, bw, bh, mA, mB, err, st); break;
                case 128: e = tma_launch<128>(g, bw, bh, mA, mB, err, st); break;
                default: e = tma_launch<256>(g, bw, bh, mA, mB, err, st); break;
            }
            lc.add(1);
            return e;
        }
    }
    if (pref <= 1) {
        int R = 0, BN = 0, smem = 0;
        if (tile_shape(g, R, BN, smem)) {
            const cudaError_t e = launch_tile(g, R, BN, smem, err, st);
            lc.add(1);
            return e;
        }
    }
    if (g.C % 8 || g.ldw % kBK || g.ldw < ((g.K + kBK - 1) / kBK) * kBK || g.K <= 0) return cudaErrorInvalidValue;
    if (g.stride != 1 && g.stride != 2) return cudaErrorInvalidValue;
    if (g.N != 16 && g.N != 32 && g.N != 64 && g.N != 128 && g.N != 256) return cudaErrorInvalidValue;
    // output columns per CTA: all N, halved while the grid would not fill the SMs (the low-resolution layers)
    const int mtiles = (g.batch * g.Ho * g.Wo + kBM - 1) / kBM;
    int bn = g.N;
    while (bn > 32 && mtiles * (g.N / bn) < 120) bn >>= 1;
    cudaError_t e;
    switch (bn) {
        case 16: e = conv_launch<16>(g, err, st); break;
        case 32: e = conv_launch<32>(g, err, st); break;
        case 64: e = conv_launch<64>(g, err, st); break;
        case 128: e = conv_launch<128>(g, err, st); break;
        case 256: e = conv_launch<256>(g, err, st); break;
        default: return cudaErrorInvalidValue;
    }
    lc.add(1);
    return e;
}

template <int BN>
static cudaError_t wgrad_launch(const WgradGemm &g, int splits, int *err, cudaStream_t st) {
    constexpr int smem = kWgStages * (kBM * kBK * 2 + BN * kBK * 2) + 1024;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_wgrad_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_wgrad_tc<BN><<<dim3(g.Mpad / kBM, splits), kThreads, smem, st>>>(g, err);
    return cudaGetLastError();
}

cudaError_t launch_wgrad_tc(const WgradGemm &g, int splits, int Cout_real, float *grad, int *err, cudaStream_t st,
                            LaunchCounter &lc) {
    {
        ProfScope _ps(lc, "conv_wgrad_tc", st);
        if (g.Cin % 8 || g.Mpad % kBM || g.Mpad < g.Kf || g.chunk % kBK) return cudaErrorInvalidValue;
        cudaError_t e;
        switch (g.Cout) {
            case 16: e = wgrad_launch<16>(g, splits, err, st); break;
            case 32: e = wgrad_launch<32>(g, splits, err, st); break;
            case 64: e = wgrad_launch<64>(g, splits, err, st); break;
            case 128: e = wgrad_launch<128>(g, splits, err, st); break;
            case 256: e = wgrad_launch<256>(g, splits, err, st); break;
            default: return cudaErrorInvalidValue;
        }
        lc.add(1);
        if (e != cudaSuccess) return e;
    }
    ProfScope _ps(lc, "wgrad_reduce", st);
    const int n = g.Kf * Cout_real;
    k_wgrad_reduce<<<(n + 255) / 256, 256, 0, st>>>(splits, g.Mpad, g.Cout, g.Kf, Cout_real, g.partial, grad);
    lc.add(1);
    return cudaGetLastError();
}

cudaError_t launch_bias_grad(int P, int C, int Creal, const void *dy, float *partial, int blocks, float *out,
                             cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "bias_grad", st);
    if (C > 256 || 256 % C) return cudaErrorInvalidValue;
    k_colsum<<<blocks, 256, 0, st>>>(P, C, static_cast<const __nv_bfloat16 *>(dy), partial);
    k_colsum_final<<<(Creal + 127) / 128, 128, 0, st>>>(blocks, C, Creal, partial, out);
    lc.add(2);
    return cudaGetLastError();
}

static int ew_blocks(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

cudaError_t launch_upsample_add_relu(int batch, int Hl, int Wl, int C, const void *t, const void *skip, void *s,
                                     cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "upsample_add", st);
    const size_t n = (size_t)batch * 4 * Hl * Wl * (C / 8);
    k_upsample_add_relu<<<ew_blocks(n), 256, 0, st>>>(batch, Hl, Wl, C, static_cast<const __nv_bfloat16 *>(t),
                                                     static_cast<const __nv_bfloat16 *>(skip),
                                                     static_cast<__nv_bfloat16 *>(s));
    lc.add(1);
    return cudaGetLastError();
}

cudaError_t launch_down_sum(int batch, int Hl, int Wl, int C, const void *ds, void *dt, cudaStream_t st,
                            LaunchCounter &lc) {
    ProfScope _ps(lc, "down_sum", st);
    const size_t n = (size_t)batch * Hl * Wl * (C / 8);
    k_down_sum<<<ew_blocks(n), 256, 0, st>>>(batch, Hl, Wl, C, static_cast<const __nv_bfloat16 *>(ds),
                                            static_cast<__nv_bfloat16 *>(dt));
    lc.add(1);
    return cudaGetLastError();
}

cudaError_t launch_output_head(int batch, int HW, int Cy, const float *y, const float *u0, const float *target,
                               float *pred, void *dy, double *loss_partial, int blocks, cudaStream_t st,
                               LaunchCounter &lc) {
    ProfScope _ps(lc, "output_head", st);
    k_output_head<<<blocks, 256, 0, st>>>(batch, HW, Cy, y, u0, target, pred, static_cast<__nv_bfloat16 *>(dy),
                                         loss_partial);
    lc.add(1);
    return cudaGetLastError();
}

cudaError_t launch_adam(size_t n, float *w, const float *grad, float *m, float *v, float lr_t, float b1, float b2,
                        float eps_t, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "adam", st);
    k_adam<<<ew_blocks(n), 256, 0, st>>>(n, w, grad, m, v, lr_t, b1, b2, eps_t);
    lc.add(1);
    return cudaGetLastError();
}

cudaError_t launch_pack_weights(int Cout, int Cst, int Cin, int taps, int Kpad, int Kdpad, const float *w, void *Wb,
                                void *Wt, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "pack_weights", st);
    const size_t n = (size_t)Cst * Kpad + (size_t)Cin * Kdpad;
    k_pack_weights<<<ew_blocks(n), 256, 0, st>>>(Cout, Cst, Cin, taps, Kpad, Kdpad, w,
                                                 static_cast<__nv_bfloat16 *>(Wb), static_cast<__nv_bfloat16 *>(Wt));
    lc.add(1);
    return cudaGetLastError();
}

}  // namespace lfrv
