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
#include "device_common.cuh"
#include "kernels.h"

namespace lfrv {

// Hole list in raster order: per-row counts, an exclusive scan over rows, per-row writes.
__global__ void k_hole_rows(int W, int H, const uint8_t *__restrict__ vis, int *__restrict__ row_count) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    int c = 0;
    for (int x = 0; x < W; ++x) c += vis[(size_t)y * W + x] ? 0 : 1;
    row_count[y] = c;
}

__global__ void k_hole_scan(int H, int *__restrict__ row_count, int *__restrict__ total) {
    // single thread: H <= 16384 rows
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int s = 0;
    for (int y = 0; y < H; ++y) {
        const int c = row_count[y];
        row_count[y] = s;
        s += c;
    }
    *total = s;
}

__global__ void k_hole_write(int W, int H, const uint8_t *__restrict__ vis, const int *__restrict__ row_start,
                             int *__restrict__ holes) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    int k = row_start[y];
    for (int x = 0; x < W; ++x)
        if (!vis[(size_t)y * W + x]) holes[k++] = y * W + x;
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
    k_hole_rows<<<(H + 127) / 128, 128, 0, st>>>(W, H, vis, row);
    k_hole_scan<<<1, 32, 0, st>>>(H, row, count);
    k_hole_write<<<(H + 127) / 128, 128, 0, st>>>(W, H, vis, row, holes);
    lc.add(3);
}

int hole_fill_partials(int nholes) { return (nholes + 255) / 256; }

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
