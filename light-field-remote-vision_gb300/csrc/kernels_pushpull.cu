// kernels_pushpull.cu -- push-pull hole filling of the IBR_color initial image on the GPU.
//
// The reference runs this on the host after copying the image down (coco_vtv_push_pull,
// sources/optimization.cu:544-651, with reduce / expand at :210-492): a pyramid of fixed height 10 is built
// by a separable 5-tap filter (a = 0.4) that ignores zero-valued samples and renormalises, visibility is
// reduced by OR, and the pyramid is expanded back writing only non-visible pixels of each level. Levels are
// W >> s by H >> s; a level with no pixels reads as zero. All three channels run in one launch (blockIdx.z).
#include "device_common.cuh"
#include "kernels.h"

namespace lfrv {

__constant__ float c_pp[5];  // {0.25 - a/2, 0.25, a, 0.25, 0.25 - a/2} computed in float

// vertical pass of reduce: in Ws x Hs -> tmp Ws x hs (value-masked, renormalised)
__global__ void k_reduce_v(int Ws, int Hs, int hs, const float *__restrict__ in, size_t in_cs,
                           float *__restrict__ tmp, size_t tmp_cs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= Ws || i >= hs) return;
    const float *p = in + blockIdx.z * in_cs;
    const int rows[5] = {max(2 * i - 2, 0), max(2 * i - 1, 0), 2 * i, min(2 * i + 1, Hs - 1), min(2 * i + 2, Hs - 1)};
    float v = 0.f, wt = 0.f;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const float s = p[(size_t)rows[k] * Ws + j];
        if (s != 0.f) {
            v += c_pp[k] * s;
            wt += c_pp[k];
        }
    }
    tmp[blockIdx.z * tmp_cs + (size_t)i * Ws + j] = (wt == 0.f) ? 0.f : v / wt;
}

// horizontal pass of reduce: tmp Ws x hs -> out ws x hs
__global__ void k_reduce_h(int Ws, int ws, int hs, const float *__restrict__ tmp, size_t tmp_cs,
                           float *__restrict__ out, size_t out_cs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= ws || i >= hs) return;
    const float *row = tmp + blockIdx.z * tmp_cs + (size_t)i * Ws;
    const int cols[5] = {max(2 * j - 2, 0), max(2 * j - 1, 0), 2 * j, min(2 * j + 1, Ws - 1), min(2 * j + 2, Ws - 1)};
    float v = 0.f, wt = 0.f;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const float s = row[cols[k]];
        if (s != 0.f) {
            v += c_pp[k] * s;
            wt += c_pp[k];
        }
    }
    out[blockIdx.z * out_cs + (size_t)i * ws + j] = (wt == 0.f) ? 0.f : v / wt;
}

// OR-reduction of the visibility (both passes fused: the 5x5 OR of the clamped window)
__global__ void k_reduce_vis(int Ws, int Hs, int ws, int hs, const uint8_t *__restrict__ in, uint8_t *__restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= ws || i >= hs) return;
    const int rows[5] = {max(2 * i - 2, 0), max(2 * i - 1, 0), 2 * i, min(2 * i + 1, Hs - 1), min(2 * i + 2, Hs - 1)};
    const int cols[5] = {max(2 * j - 2, 0), max(2 * j - 1, 0), 2 * j, min(2 * j + 1, Ws - 1), min(2 * j + 2, Ws - 1)};
    uint8_t any = 0;
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
        for (int b = 0; b < 5; ++b) any |= in[(size_t)rows[a] * Ws + cols[b]];
    out[(size_t)i * ws + j] = any ? 1 : 0;
}

// vertical pass of expand: in ws x hs (level s) -> tmp ws x Hs; an empty level reads as 0
__global__ void k_expand_v(int Hs, int ws, int hs, const float *__restrict__ in, size_t in_cs,
                           float *__restrict__ tmp, size_t tmp_cs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= ws || i >= Hs) return;
    const float *p = in + blockIdx.z * in_cs;
    // Rows past the coarser level (odd sizes) are clamped to its last row; the reference reads beyond its
    // array there (sources/optimization.cu:447-452).
    auto at = [&](int r) { return (hs > 0) ? p[(size_t)min(r, hs - 1) * ws + j] : 0.f; };
    float v = 0.f;
    if (i % 2 == 0) {
        v += 2.f * c_pp[0] * (((i - 2) / 2 < 0) ? at(0) : at((i - 2) / 2));
        v += 2.f * c_pp[2] * at(i / 2);
        v += 2.f * c_pp[4] * ((hs - 1 < (i + 2) / 2) ? at(hs - 1) : at((i + 2) / 2));
    } else {
        v += 2.f * c_pp[1] * (((i - 1) / 2 < 0) ? at(0) : at((i - 1) / 2));
        v += 2.f * c_pp[3] * ((hs - 1 < (i + 1) / 2) ? at(hs - 1) : at((i + 1) / 2));
    }
    tmp[blockIdx.z * tmp_cs + (size_t)i * ws + j] = v;
}

// horizontal pass of expand: tmp ws x Hs -> out Ws x Hs at non-visible pixels
__global__ void k_expand_h(int Ws, int Hs, int ws, const float *__restrict__ tmp, size_t tmp_cs,
                           float *__restrict__ out, size_t out_cs, const uint8_t *__restrict__ vis) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= Ws || i >= Hs) return;
    if (vis[(size_t)i * Ws + j]) return;
    const float *row = tmp + blockIdx.z * tmp_cs + (size_t)i * ws;
    auto at = [&](int c) { return (ws > 0) ? row[min(c, ws - 1)] : 0.f; };
    float v = 0.f;
    if (j % 2 == 0) {
        v += 2.f * c_pp[0] * (((j - 2) / 2 < 0) ? at(0) : at((j - 2) / 2));
        v += 2.f * c_pp[2] * at(j / 2);
        v += 2.f * c_pp[4] * ((ws - 1 < (j + 2) / 2) ? at(ws - 1) : at((j + 2) / 2));
    } else {
        v += 2.f * c_pp[1] * (((j - 1) / 2 < 0) ? at(0) : at((j - 1) / 2));
        v += 2.f * c_pp[3] * ((ws - 1 < (j + 1) / 2) ? at(ws - 1) : at((j + 1) / 2));
    }
    out[blockIdx.z * out_cs + (size_t)i * Ws + j] = v;
}

__global__ void k_pp_finish(size_t N3, const float *__restrict__ filled, const float *__restrict__ orig, int faithful,
                            float *__restrict__ U) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N3) return;
    U[i] = faithful ? filled[i] - orig[i] : filled[i];
}

void launch_push_pull(int W, int H, bool faithful, const uint8_t *vis, float *U, PushPull &pp, cudaStream_t st,
                      LaunchCounter &lc) {
    ProfScope _ps(lc, "push_pull", st);
    static bool init = false;
    if (!init) {
        const float a = 0.4f;
        const float k[5] = {0.25f - 0.5f * a, 0.25f, a, 0.25f, 0.25f - 0.5f * a};
        cudaMemcpyToSymbol(c_pp, k, sizeof(k));
        init = true;
    }
    const int height = 10;
    const size_t N = (size_t)W * H;
    cudaMemcpyAsync(pp.orig, U, 3 * N * sizeof(float), cudaMemcpyDeviceToDevice, st);
    // level 0 of the pyramid is U itself (updated in place by the final expand)
    pp.img[0] = U;
    cudaMemcpyAsync(pp.vis[0], vis, N, cudaMemcpyDeviceToDevice, st);
    const dim3 b(32, 8);
    auto g3 = [&](int x, int y) { return dim3((x + 31) / 32, (y + 7) / 8, 3); };
    auto g1 = [&](int x, int y) { return dim3((x + 31) / 32, (y + 7) / 8, 1); };
    for (int s = 1; s <= height; ++s) {
        const int Ws = W >> (s - 1), Hs = H >> (s - 1), ws = W >> s, hs = H >> s;
        if (ws <= 0 || hs <= 0) continue;
        const size_t cs_in = (size_t)Ws * Hs, cs_tmp = (size_t)Ws * hs, cs_out = (size_t)ws * hs;
        k_reduce_v<<<g3(Ws, hs), b, 0, st>>>(Ws, Hs, hs, pp.img[s - 1], cs_in, pp.tmp, cs_tmp);
        k_reduce_h<<<g3(ws, hs), b, 0, st>>>(Ws, ws, hs, pp.tmp, cs_tmp, pp.img[s], cs_out);
        k_reduce_vis<<<g1(ws, hs), b, 0, st>>>(Ws, Hs, ws, hs, pp.vis[s - 1], pp.vis[s]);
        lc.add(3);
    }
    for (int s = height; s > 0; --s) {
        const int Ws = W >> (s - 1), Hs = H >> (s - 1), ws = W >> s, hs = H >> s;
        if (Ws <= 0 || Hs <= 0) continue;
        const int wse = (ws > 0 && hs > 0) ? ws : 0, hse = (ws > 0 && hs > 0) ? hs : 0;
        const size_t cs_in = (size_t)wse * hse, cs_tmp = (size_t)ws * Hs, cs_out = (size_t)Ws * Hs;
        if (ws > 0) {
            k_expand_v<<<g3(ws, Hs), b, 0, st>>>(Hs, ws, hse, pp.img[s], cs_in, pp.tmp, cs_tmp);
            lc.add(1);
        }
        k_expand_h<<<g3(Ws, Hs), b, 0, st>>>(Ws, Hs, ws, pp.tmp, cs_tmp, pp.img[s - 1], cs_out, pp.vis[s - 1]);
        lc.add(1);
    }
    k_pp_finish<<<(unsigned)((3 * N + 255) / 256), 256, 0, st>>>(3 * N, U, pp.orig, faithful ? 1 : 0, U);
    lc.add(1);
}

}  // namespace lfrv
