// kernels_warp.cu -- warp stage: target depth map, tau warps, dtau/dz (sm_103a).
//
// Restates the GL pipeline of the reference's warp exporter as CUDA kernels writing device buffers:
//   target depth map: Scene::computeTargetDepthMap (sources/openGL/scene.cpp:1506-1544) drawing
//     depthSplatting.{vert,geom,frag}: each input pixel becomes a tilted quad, rasterised into the target
//     with a depth test; the colour written is the quad centre's target depth;
//   tau: tauWarp.frag:25-74 (projection, deformation weight capped at 30, visibility codes -2 / -1 with a
//     0.10 depth tolerance against the bilinearly sampled target depth map);
//   dtau/dz: tauPartial.frag:23-48 (sigma_z = 10 in channel 0).
// Per input view the host folds the cameras into M = K_u R_u R_k^T K_k^-1 and b = K_u (t_u - R_u R_k^T t_k),
// so the target homogeneous point of input pixel (x, y) at depth z is x_h = M (z (x, y, 1)) + b.
#include <algorithm>
#include <type_traits>
#include "device_common.cuh"
#include "kernels.h"

namespace lfrv {

__device__ __forceinline__ void mv3(const float *M, float x, float y, float z, float *o) {
    o[0] = M[0] * x + M[1] * y + M[2] * z;
    o[1] = M[3] * x + M[4] * y + M[5] * z;
    o[2] = M[6] * x + M[7] * y + M[8] * z;
}

// One input view's fold of the cameras: the target homogeneous point of pixel (x, y) at depth z is M (z x, z y, z) + b.
struct ViewCam {
    float M[9], b[3];
};

__device__ __forceinline__ ViewCam view_cam(const WarpCams &cams, int v) {
    ViewCam c;
#pragma unroll
    for (int i = 0; i < 9; ++i) c.M[i] = cams.M[v][i];
#pragma unroll
    for (int i = 0; i < 3; ++i) c.b[i] = cams.b[v][i];
    return c;
}

// ------------------------------------------------------------------ target depth map
__device__ __forceinline__ float edgef(float ax, float ay, float bx, float by, float px, float py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
__device__ __forceinline__ bool top_left(float ax, float ay, float bx, float by, bool ccw) {
    const float ex = bx - ax, ey = by - ay;
    if (!ccw) return (ey == 0.f && ex < 0.f) || ey > 0.f;
    return (ey == 0.f && ex > 0.f) || ey < 0.f;
}

// Covered pixel centres of a triangle keep the largest interpolated 1/z (nearest surface); ties keep the
// smaller centre depth. Key = (bits(1/z) << 32) | (~bits(z_centre)), both positive floats.
__device__ __forceinline__ void depth_test(int x, int y, int W, float iz, unsigned int zlow,
                                           unsigned long long *zkey) {
    if (!(iz > 0.f)) return;
    const unsigned long long key = ((unsigned long long)__float_as_uint(iz) << 32) | zlow;
    unsigned long long *slot = zkey + (size_t)y * W + x;
    // keys only grow: a candidate already beaten needs no atomic
    if (__ldcg(slot) < key) atomicMax(slot, key);
}

// Set-up of one triangle of the strip: orientation, top-left flags of its edges (v1v2, v2v0, v0v1) and its
// clipped bounding box; live is false for zero area, an empty box, or a box wider than 64 pixels
// (degenerate, grazing quads are skipped).
struct TriSetup {
    bool live, tl0, tl1, tl2;
    float sgn;  // +1 counter-clockwise, -1 clockwise: edge values are multiplied by it
    int xmin, xmax, ymin, ymax;
};

__device__ __forceinline__ TriSetup tri_setup(const float *v0, const float *v1, const float *v2, int W, int H) {
    TriSetup t;
    t.live = false;
    const float area = edgef(v0[0], v0[1], v1[0], v1[1], v2[0], v2[1]);
    if (area == 0.f) return t;
    const bool ccw = area > 0.f;
    t.sgn = ccw ? 1.f : -1.f;
    // a pixel centre x + 1/2 can lie in the triangle only when min <= x + 1/2 <= max
    const float x_lo = fminf(v0[0], fminf(v1[0], v2[0])), x_hi = fmaxf(v0[0], fmaxf(v1[0], v2[0]));
    const float y_lo = fminf(v0[1], fminf(v1[1], v2[1])), y_hi = fmaxf(v0[1], fmaxf(v1[1], v2[1]));
    // grazing triangles wider than 64 pixels are skipped, measured on the conservative clipped box
    {
        const int cx0 = max(0, (int)floorf(x_lo - 0.5f)), cx1 = min(W - 1, (int)ceilf(x_hi - 0.5f));
        const int cy0 = max(0, (int)floorf(y_lo - 0.5f)), cy1 = min(H - 1, (int)ceilf(y_hi - 0.5f));
        if (cx1 < cx0 || cy1 < cy0 || cx1 - cx0 > 64 || cy1 - cy0 > 64) return t;
    }
    t.xmin = max(0, (int)ceilf(x_lo - 0.5f));
    t.xmax = min(W - 1, (int)floorf(x_hi - 0.5f));
    t.ymin = max(0, (int)ceilf(y_lo - 0.5f));
    t.ymax = min(H - 1, (int)floorf(y_hi - 0.5f));
    if (t.xmax < t.xmin || t.ymax < t.ymin) return t;
    t.tl0 = top_left(v1[0], v1[1], v2[0], v2[1], ccw);
    t.tl1 = top_left(v2[0], v2[1], v0[0], v0[1], ccw);
    t.tl2 = top_left(v0[0], v0[1], v1[0], v1[1], ccw);
    t.live = true;
    return t;
}

// Coverage test of a pixel centre given the three (unsigned) edge values; on success iz is the interpolated
// 1/z of the triangle (w0 v0 + w1 v1 + w2 v2) / (w0 + w1 + w2).
__device__ __forceinline__ bool tri_cover(const TriSetup &t, float e0, float e1, float e2, float z0, float z1,
                                          float z2, float &iz) {
    const float w0 = t.sgn * e0, w1 = t.sgn * e1, w2 = t.sgn * e2;
    if (w0 < 0.f || w1 < 0.f || w2 < 0.f) return false;
    if ((w0 == 0.f && !t.tl0) || (w1 == 0.f && !t.tl1) || (w2 == 0.f && !t.tl2)) return false;
    const float s = w0 + w1 + w2;
    iz = (w0 * z0 + w1 * z1 + w2 * z2) / s;
    return true;
}

// The quad (strip BL v0, TL v1, BR v2, TR v3) as triangles A = (v0, v1, v2) and B = (v1, v2, v3), which share
// the edge v1v2 (A's edge 0, B's edge 2). One pass over the union of their boxes evaluates that edge once per
// pixel; each triangle's coverage and depth are those of rasterising it alone. The box's pixels are taken
// first, first + stride, ... in row-major order (a warp shares one quad with first = lane, stride = 32; the
// depth test's result does not depend on the order).
__device__ void raster_quad(const float (*v)[3], float zc, int W, int H, unsigned long long *zkey, int first = 0,
                            int stride = 1) {
    const TriSetup A = tri_setup(v[0], v[1], v[2], W, H), B = tri_setup(v[1], v[2], v[3], W, H);
    if (!A.live && !B.live) return;
    const int xmin = A.live ? (B.live ? min(A.xmin, B.xmin) : A.xmin) : B.xmin;
    const int xmax = A.live ? (B.live ? max(A.xmax, B.xmax) : A.xmax) : B.xmax;
    const int ymin = A.live ? (B.live ? min(A.ymin, B.ymin) : A.ymin) : B.ymin;
    const int ymax = A.live ? (B.live ? max(A.ymax, B.ymax) : A.ymax) : B.ymax;
    const unsigned int zlow = ~__float_as_uint(zc);
    const int bw = xmax - xmin + 1, npx = bw * (ymax - ymin + 1);
    if (A.live && B.live && A.sgn != B.sgn) {
        // Opposite windings (a strip quad that does not fold): the shared edge splits the quad, and a pixel
        // centre on the edge belongs to the triangle whose edge is top-left (the two flags are complementary),
        // so only the triangle on the pixel's side is tested. With o = v0 (A) or v3 (B), its other edges are
        // v2 -> o and o -> v1, and its depth (e12 z_o + e2o z_1 + eo1 z_2) / (e12 + e2o + eo1) equals
        // tri_cover's (the winding sign cancels in the quotient).
        for (int p = first; p < npx; p += stride) {
                const int y = ymin + p / bw, x = xmin + p % bw;
                const float px = x + 0.5f, py = y + 0.5f;
                const float e12 = edgef(v[1][0], v[1][1], v[2][0], v[2][1], px, py);
                const float a12 = A.sgn * e12;
                const bool inA = a12 > 0.f || (a12 == 0.f && A.tl0);
                const float ox = inA ? v[0][0] : v[3][0], oy = inA ? v[0][1] : v[3][1];
                const float oz = inA ? v[0][2] : v[3][2], sg = inA ? A.sgn : B.sgn;
                const bool tla = inA ? A.tl1 : B.tl0, tlb = inA ? A.tl2 : B.tl1;
                const float ea = edgef(v[2][0], v[2][1], ox, oy, px, py);
                const float eb = edgef(ox, oy, v[1][0], v[1][1], px, py);
                const float wa = sg * ea, wb = sg * eb;
                if (wa < 0.f || wb < 0.f || (wa == 0.f && !tla) || (wb == 0.f && !tlb)) continue;
                const float w0 = sg * e12;
                const float iz = (w0 * oz + wa * v[1][2] + wb * v[2][2]) / (w0 + wa + wb);
                depth_test(x, y, W, iz, zlow, zkey);
            }
        return;
    }
    for (int p = first; p < npx; p += stride) {
            const int y = ymin + p / bw, x = xmin + p % bw;
            const float px = x + 0.5f, py = y + 0.5f;
            const float e12 = edgef(v[1][0], v[1][1], v[2][0], v[2][1], px, py);
            float iz;
            if (A.live && A.sgn * e12 >= 0.f &&
                tri_cover(A, e12, edgef(v[2][0], v[2][1], v[0][0], v[0][1], px, py),
                          edgef(v[0][0], v[0][1], v[1][0], v[1][1], px, py), v[0][2], v[1][2], v[2][2], iz))
                depth_test(x, y, W, iz, zlow, zkey);
            if (B.live && B.sgn * e12 >= 0.f &&
                tri_cover(B, edgef(v[2][0], v[2][1], v[3][0], v[3][1], px, py),
                          edgef(v[3][0], v[3][1], v[1][0], v[1][1], px, py), e12, v[1][2], v[2][2], v[3][2], iz))
                depth_test(x, y, W, iz, zlow, zkey);
        }
}

// raster_quad for the common quad: its two triangles have opposite windings (the strip does not fold) and its
// box holds at most 3 x 3 pixel centres. Coverage and depth are tri_cover's for each triangle:
//   - a centre is tested against the triangle on its side of the shared edge v1v2 only (a centre on that edge
//     belongs to the triangle for which the edge is top-left; the two flags are complementary);
//   - edge values are affine in the centre's offset (i, j) from the box's first centre: each edge keeps its
//     value there and its steps along i and j, scaled by the triangle's winding sign, so "inside" is w >= thr
//     on every edge, with thr = 0 on a top-left edge and the smallest positive float elsewhere (the library
//     is built without flush-to-zero). A row's values are its base plus the column steps;
//   - the depth is the triangle's 1/z plane (tri_cover's barycentric interpolation, which is affine over the
//     triangle) evaluated at the centre the same way; it differs from tri_cover's quotient by float rounding
//     only.
// The window is unrolled at 2 x 2 or 3 x 3. Returns false when the quad needs raster_quad.
__device__ __forceinline__ bool raster_quad_small(const float (*v)[3], float zc, int W, int H,
                                                  unsigned long long *zkey) {
    const float areaA = edgef(v[0][0], v[0][1], v[1][0], v[1][1], v[2][0], v[2][1]);
    const float areaB = edgef(v[1][0], v[1][1], v[2][0], v[2][1], v[3][0], v[3][1]);
    if (!(areaA != 0.f && areaB != 0.f && ((areaA > 0.f) != (areaB > 0.f)))) return false;
    const float x_lo = fminf(fminf(v[0][0], v[1][0]), fminf(v[2][0], v[3][0]));
    const float x_hi = fmaxf(fmaxf(v[0][0], v[1][0]), fmaxf(v[2][0], v[3][0]));
    const float y_lo = fminf(fminf(v[0][1], v[1][1]), fminf(v[2][1], v[3][1]));
    const float y_hi = fmaxf(fmaxf(v[0][1], v[1][1]), fmaxf(v[2][1], v[3][1]));
    const int xmin = max(0, (int)ceilf(x_lo - 0.5f)), xmax = min(W - 1, (int)floorf(x_hi - 0.5f));
    const int ymin = max(0, (int)ceilf(y_lo - 0.5f)), ymax = min(H - 1, (int)floorf(y_hi - 0.5f));
    if (xmax < xmin || ymax < ymin) return true;  // no pixel centre in the box
    if (xmax - xmin > 2 || ymax - ymin > 2) return false;
    const float ox = (float)xmin + 0.5f, oy = (float)ymin + 0.5f;
    float qx[4], qy[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        qx[k] = v[k][0] - ox;
        qy[k] = v[k][1] - oy;
    }
    const bool ccwA = areaA > 0.f;
    const float sA = ccwA ? 1.f : -1.f;
    constexpr float kTiny = 1.40129846e-45f;  // smallest positive float: w >= kTiny is w > 0
    // edge a -> b scaled by s: w(i, j) = (s dx)(j - qy[a]) - (s dy)(i - qx[a]) = c0 + gi i + gj j
    struct Edge {
        float c0, gi, gj, thr;
    };
    auto edge = [&](int a, int b, float s, bool ccw) {
        Edge e;
        const float dx = s * (qx[b] - qx[a]), dy = s * (qy[b] - qy[a]);
        e.c0 = dy * qx[a] - dx * qy[a];
        e.gi = -dy;
        e.gj = dx;
        e.thr = top_left(qx[a], qy[a], qx[b], qy[b], ccw) ? 0.f : kTiny;
        return e;
    };
    const Edge e12 = edge(1, 2, sA, ccwA), a1 = edge(2, 0, sA, ccwA), a2 = edge(0, 1, sA, ccwA);
    const Edge b0 = edge(2, 3, -sA, !ccwA), b1 = edge(3, 1, -sA, !ccwA);
    // 1/z is affine over each triangle: iz(i, j) = P0 + Pi i + Pj j, from the barycentric numerator (the edge
    // values weighting the vertices' 1/z) over the triangle's doubled area (the sum of its sign-scaled edge
    // values)
    auto plane = [&](const Edge &e0, float za, const Edge &e1, float zb, const Edge &e2, float zc2, float s0,
                     float area) {
        const float inv = __fdividef(1.0f, fabsf(area));
        Edge p;
        p.c0 = (s0 * e0.c0 * za + e1.c0 * zb + e2.c0 * zc2) * inv;
        p.gi = (s0 * e0.gi * za + e1.gi * zb + e2.gi * zc2) * inv;
        p.gj = (s0 * e0.gj * za + e1.gj * zb + e2.gj * zc2) * inv;
        p.thr = 0.f;
        return p;
    };
    // A = (v0, v1, v2): weights (w12, wa1, wa2); B = (v1, v2, v3): weights (wb0, wb1, -w12)
    const Edge pA = plane(e12, v[0][2], a1, v[1][2], a2, v[2][2], 1.f, areaA);
    const Edge pB = plane(e12, v[3][2], b0, v[1][2], b1, v[2][2], -1.f, areaB);
    const unsigned int zlow = ~__float_as_uint(zc);
    // value of an affine function at row base r (its value at (0, j)) stepped i columns
    auto at = [](const Edge &e, float r, int i) { return i == 0 ? r : fmaf(e.gi, (float)i, r); };
    // one row of the window at a time: the cells' keys, then their depth-buffer loads together (the depth test of
    // depth_test, its loads not serialised behind each other's branches). The window is unrolled at its size: 2 x 2
    // (the common box of a quad at twice the input resolution) or 3 x 3; each cell's values are the same either way
    auto window = [&](auto nx_c) {
        constexpr int NX = decltype(nx_c)::value;
#pragma unroll
        for (int j = 0; j < NX; ++j) {
            if (j > ymax - ymin) break;
            unsigned long long *row = zkey + (size_t)(ymin + j) * W + xmin;
            auto base = [j](const Edge &e) { return j == 0 ? e.c0 : fmaf(e.gj, (float)j, e.c0); };
            const float r12 = base(e12), ra1 = base(a1), ra2 = base(a2), rb0 = base(b0), rb1 = base(b1);
            const float rA = base(pA), rB = base(pB);
            unsigned long long key[NX], cur[NX];
            bool hit[NX];
#pragma unroll
            for (int i = 0; i < NX; ++i) {
                const float w12 = at(e12, r12, i);
                const bool inA = w12 >= e12.thr;
                const float wa1 = at(a1, ra1, i), wa2 = at(a2, ra2, i), wb0 = at(b0, rb0, i), wb1 = at(b1, rb1, i);
                const bool cov = inA ? (wa1 >= a1.thr && wa2 >= a2.thr) : (wb0 >= b0.thr && wb1 >= b1.thr);
                const float iz = inA ? at(pA, rA, i) : at(pB, rB, i);
                hit[i] = i <= xmax - xmin && cov && iz > 0.f;
                key[i] = ((unsigned long long)__float_as_uint(iz) << 32) | zlow;
            }
#pragma unroll
            for (int i = 0; i < NX; ++i) cur[i] = hit[i] ? __ldcg(row + i) : ~0ull;
#pragma unroll
            for (int i = 0; i < NX; ++i)
                if (hit[i] && cur[i] < key[i]) atomicMax(row + i, key[i]);
        }
    };
    if (xmax - xmin <= 1 && ymax - ymin <= 1) window(std::integral_constant<int, 2>{});
    else window(std::integral_constant<int, 3>{});
    return true;
}

// The tilted quad of input pixel m of view cam c in target pixel space: its corners (x, y, 1/w) in strip order
// BL, TL, BR, TR and its centre depth zc. False when the pixel is not splatted (invalid depth, or a corner behind
// the near plane).
__device__ __forceinline__ bool zsplat_vertices(const ViewCam &c, int m, int w, int n, float rw, float z, float zx,
                                                float zy, float (*vert)[3], float &zc) {
    if (z >= 1000.0f * 0.5f) return false;  // INVALID_DEPTH / 2 (depthSplatting.geom:21)
    int px, py;
    pixel_of(m, w, n, rw, px, py);
    const float cx = px + 0.5f, cy = py + 0.5f;
    // x_h is linear in the pixel-space point scaled by its depth: with q = M (cx, cy, 1), the centre maps to
    // z q + b and the corner (cx + dx, cy + dy) at depth z + dx zx + dy zy to (z + dx zx + dy zy)(q + dx M_0 +
    // dy M_1) + b, M_0 and M_1 the first two columns of M
    float q[3];
    mv3(c.M, cx, cy, 1.f, q);
    zc = fmaf(z, q[2], c.b[2]);
    const float off[4][2] = {{-0.5f, -0.5f}, {-0.5f, 0.5f}, {0.5f, -0.5f}, {0.5f, 0.5f}};  // BL TL BR TR
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float dx = off[k][0], dy = off[k][1];
        const float zk = fmaf(dy, zy, fmaf(dx, zx, z));
        float xh[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) xh[r] = fmaf(zk, fmaf(dy, c.M[3 * r + 1], fmaf(dx, c.M[3 * r], q[r])), c.b[r]);
        if (!(xh[2] > 1e-2f)) return false;  // behind the near plane (zNear = 1e-2, sources/pinholeCamera.cpp:133)
        const float iw = __fdividef(1.0f, xh[2]);  // approximate reciprocal: vertex positions within 2 ulp
        vert[k][0] = xh[0] * iw;
        vert[k][1] = xh[1] * iw;
        vert[k][2] = iw;
    }
    return true;
}

// Queue of the quads that need the general rasteriser (a box beyond 3 x 3 pixel centres, or a folded strip):
// word 0 counts them, entries (view << 24 | pixel) follow from word kZdeferHead. Those quads are few but their
// boxes are large, so one lane rasterising one of them would hold its whole warp; k_zsplat_defer gives each a
// warp. When the queue is full the quad is rasterised where it is.
constexpr int kZdeferHead = 32;
struct ZDefer {
    unsigned int *q;
    unsigned int cap;
};

// One input pixel m of view v (camera c): its tilted quad into the depth buffer.
__device__ __forceinline__ void zsplat_pixel(const ViewCam &c, int v, int m, int w, int n, float rw, float z, float zx,
                                             float zy, int W, int H, unsigned long long *zkey, ZDefer defer) {
    float vert[4][3], zc;
    if (!zsplat_vertices(c, m, w, n, rw, z, zx, zy, vert, zc)) return;
    if (raster_quad_small(vert, zc, W, H, zkey)) return;
    const unsigned int slot = defer.q ? atomicAdd(defer.q, 1u) : defer.cap;
    if (slot < defer.cap) defer.q[kZdeferHead + slot] = ((unsigned int)v << 24) | (unsigned int)m;
    else raster_quad(vert, zc, W, H, zkey);
}

// Two input pixels per thread (m and m + blockDim.x): the second pixel's depth is loaded before the first is
// rasterised, so its latency hides behind that work.
constexpr int kZsplatPerThread = 2;

__global__ void __launch_bounds__(256, 4) k_zsplat(int V, int w, int h, const float *__restrict__ depth,
                                                const WarpCams cams, int W, int H,
                                                unsigned long long *__restrict__ zkey, ZDefer defer) {
    pdl_trigger();  // k_tau, launched next, waits for this grid's completion
    const int m0 = blockIdx.x * blockDim.x * kZsplatPerThread + threadIdx.x, m1 = m0 + blockDim.x;
    const int v = blockIdx.y;
    const int n = w * h;
    if (m0 >= n) return;
    const float *dz = depth + (size_t)v * 3 * n;
    const float z0 = dz[m0], zx0 = dz[n + m0], zy0 = dz[2 * n + m0];
    float z1 = 0.f, zx1 = 0.f, zy1 = 0.f;
    if (m1 < n) z1 = dz[m1], zx1 = dz[n + m1], zy1 = dz[2 * n + m1];
    const ViewCam c = view_cam(cams, v);
    const float rw = __frcp_rn((float)w);
    zsplat_pixel(c, v, m0, w, n, rw, z0, zx0, zy0, W, H, zkey, defer);
    if (m1 < n) zsplat_pixel(c, v, m1, w, n, rw, z1, zx1, zy1, W, H, zkey, defer);
}

// The queued quads of k_zsplat, one warp each: the corners again (the same arithmetic), then the lanes share
// the general rasteriser's box.
__global__ void __launch_bounds__(256) k_zsplat_defer(int w, int h, const float *__restrict__ depth,
                                                     const WarpCams cams, int W, int H,
                                                     unsigned long long *__restrict__ zkey, ZDefer defer) {
    pdl_wait();
    pdl_trigger();
    const unsigned int cnt = min(__ldcg(defer.q), defer.cap);
    const int lane = threadIdx.x & 31;
    const unsigned int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = w * h;
    const float rw = __frcp_rn((float)w);
    for (unsigned int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < cnt; it += nw) {
        const unsigned int e = __ldcg(defer.q + kZdeferHead + it);
        const int v = (int)(e >> 24), m = (int)(e & 0xFFFFFFu);
        const float *dz = depth + (size_t)v * 3 * n;
        float vert[4][3], zc;
        if (!zsplat_vertices(view_cam(cams, v), m, w, n, rw, __ldg(dz + m), __ldg(dz + n + m), __ldg(dz + 2 * n + m),
                             vert, zc))
            continue;
        raster_quad(vert, zc, W, H, zkey, lane, 32);
    }
}

// The target depth a z-buffer key holds (its centre depth; 0 where nothing was splatted).
__device__ __forceinline__ float zkey_depth(unsigned long long k) {
    return k ? __uint_as_float(~(unsigned int)(k & 0xFFFFFFFFull)) : 0.0f;
}

__global__ void k_zresolve(size_t N, const unsigned long long *__restrict__ zkey, float *__restrict__ zbuf) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    zbuf[i] = zkey_depth(zkey[i]);
}

// ------------------------------------------------------------------ tau and dtau/dz
// GL_LINEAR on a sampler2DRect with CLAMP_TO_EDGE (sources/openGL/texture.cpp:153-156) of the target depth map,
// read from the resolved map or straight from the z-buffer keys (zkey_depth of each tap).
__device__ __forceinline__ float bilinear_clamp(const unsigned long long *zkey, int W, int H, float u, float v) {
    const float fx = u - 0.5f, fy = v - 0.5f;
    const float flx = floorf(fx), fly = floorf(fy);
    const float ax = fx - flx, ay = fy - fly;
    const int x0 = (int)flx, y0 = (int)fly;
    auto at = [&](int x, int y) {
        x = min(max(x, 0), W - 1);
        y = min(max(y, 0), H - 1);
        return zkey_depth(__ldg(zkey + (size_t)y * W + x));
    };
    return (1.f - ay) * ((1.f - ax) * at(x0, y0) + ax * at(x0 + 1, y0)) +
           ay * ((1.f - ax) * at(x0, y0 + 1) + ax * at(x0 + 1, y0 + 1));
}
__device__ __forceinline__ float bilinear_clamp(const float *img, int W, int H, float u, float v) {
    const float fx = u - 0.5f, fy = v - 0.5f;
    const float flx = floorf(fx), fly = floorf(fy);
    const float ax = fx - flx, ay = fy - fly;
    const int x0 = (int)flx, y0 = (int)fly;
    auto at = [&](int x, int y) {
        x = min(max(x, 0), W - 1);
        y = min(max(y, 0), H - 1);
        return __ldg(img + (size_t)y * W + x);
    };
    return (1.f - ay) * ((1.f - ax) * at(x0, y0) + ax * at(x0 + 1, y0)) +
           ay * ((1.f - ax) * at(x0, y0 + 1) + ax * at(x0 + 1, y0 + 1));
}

// k_tau takes kTauPer source pixels per thread (m, m + blockDim.x): both are projected, then both bilinear
// samples of the target depth map are issued, then both are finished, so the dependent loads overlap.
constexpr int kTauPer = 2;

struct TauPix {
    float z, xu, yu, zt, deform, rx, ry;  // zt: the point's depth in the target camera
};

__device__ __forceinline__ TauPix tau_project(const ViewCam &c, int m, int w, int n, float rw, float z, float zx,
                                              float zy) {
    TauPix p;
    p.z = z;
    int px, py;
    pixel_of(m, w, n, rw, px, py);
    const float x = px + 0.5f, y = py + 0.5f;
    // with mk = M (x, y, 1): x_h = z mk + b, and the Jacobian's columns M (x zx + z, y zx, zx) = zx mk + z M_0
    // and M (x zy, y zy + z, zy) = zy mk + z M_1 (M_0, M_1 the first two columns of M)
    float mk[3], xuh[3], m0[3], m1[3];
    mv3(c.M, x, y, 1.0f, mk);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        xuh[r] = fmaf(z, mk[r], c.b[r]);
        m0[r] = fmaf(zx, mk[r], z * c.M[3 * r]);
        m1[r] = fmaf(zy, mk[r], z * c.M[3 * r + 1]);
    }
    p.xu = 0.f;
    p.yu = 0.f;
    if (xuh[2] != 0.f) {
        p.xu = xuh[0] / xuh[2];
        p.yu = xuh[1] / xuh[2];
    }
    p.zt = xuh[2];
    // Jacobian of the euclidean normalisation applied to M columns (tauWarp.frag:41-50)
    const float iz = 1.0f / xuh[2];
    const float d00 = (m0[0] - p.xu * m0[2]) * iz, d01 = (m0[1] - p.yu * m0[2]) * iz;
    const float d10 = (m1[0] - p.xu * m1[2]) * iz, d11 = (m1[1] - p.yu * m1[2]) * iz;
    p.deform = 1.0f / fabsf(d00 * d11 - d01 * d10);
    if (p.deform >= 30.0f) p.deform = 30.0f;
    p.rx = (mk[0] - p.xu * mk[2]) * iz;
    p.ry = (mk[1] - p.yu * mk[2]) * iz;
    return p;
}

__global__ void __launch_bounds__(256) k_tau(int V, int w, int h, const float *__restrict__ depth,
                                             const WarpCams cams, int W, int H,
                                             const float *__restrict__ zbuf, float *__restrict__ tau3,
                                             float *__restrict__ dpart3, float *__restrict__ tau2,
                                             float *__restrict__ dp2, BucketCount bc,
                                             const unsigned long long *__restrict__ zkey) {
    pdl_wait();
    pdl_trigger();
    // views vary fastest along the grid: the blocks in flight cover one band of source rows in every view, so
    // the inverse map's counters they update stay in one band of the target (and in L2)
    const int v = (int)(blockIdx.x % (unsigned)V);
    const int n = w * h;
    const int m0 = (int)(blockIdx.x / (unsigned)V) * blockDim.x * kTauPer + threadIdx.x;
    if (m0 >= n) return;
    const float *dz = depth + (size_t)v * 3 * n;
    const ViewCam c = view_cam(cams, v);
    const float rw = __frcp_rn((float)w);
    TauPix px[kTauPer];
    float zs[kTauPer];
#pragma unroll
    for (int j = 0; j < kTauPer; ++j) {
        const int m = min(m0 + j * (int)blockDim.x, n - 1);
        px[j] = tau_project(c, m, w, n, rw, dz[m], dz[n + m], dz[2 * n + m]);
    }
    // the target depth map at every projection (clamped, so every sample is in bounds; out-of-range points
    // do not use it)
#pragma unroll
    for (int j = 0; j < kTauPer; ++j)
        zs[j] = zbuf ? bilinear_clamp(zbuf, W, H, px[j].xu, px[j].yu) : bilinear_clamp(zkey, W, H, px[j].xu, px[j].yu);
#pragma unroll
    for (int j = 0; j < kTauPer; ++j) {
        const int m = m0 + j * (int)blockDim.x;
        if (m >= n) break;
        const TauPix &p = px[j];
        float t0, t1, t2;
        if (p.xu <= 0.f || (float)W <= p.xu || p.yu <= 0.f || (float)H <= p.yu || p.z >= 500.0f) {
            t0 = -2.0f;
            t1 = -2.0f;
            t2 = 0.0f;
        } else if (p.zt > zs[j] + 0.10f) {
            t0 = -1.0f;
            t1 = -1.0f;
            t2 = 0.0f;
        } else {
            t0 = p.xu;
            t1 = p.yu;
            t2 = p.deform;
        }
        const size_t b3 = (size_t)v * 3 * n, b2 = (size_t)v * 2 * n;
        if (tau3) {
            tau3[b3 + m] = t0;
            tau3[b3 + n + m] = t1;
            tau3[b3 + 2 * n + m] = t2;
        }
        if (dpart3) {
            dpart3[b3 + m] = 10.0f;
            dpart3[b3 + n + m] = p.rx;
            dpart3[b3 + 2 * n + m] = p.ry;
        }
        if (tau2) {
            tau2[b2 + m] = t0;
            tau2[b2 + n + m] = t1;
        }
        if (dp2) {
            dp2[b2 + m] = 10.0f * p.rx;
            dp2[b2 + n + m] = 10.0f * p.ry;
        }
        // the inverse map's count of this pixel's bucket, from the tau just written (k_bucket_count's rule)
        if (bc.count) {
            const long long b = bucket_of(t0, t1, W, H, bc.dsf, bc.BW);
            if (b >= 0) {
                atomicAdd(&bc.count[b], 1u);
                if (bc.mask) atomicOr(&bc.mask[(size_t)(v >> 6) * bc.nb + b], 1ull << (v & 63));
            }
        }
    }
}

void launch_zbuffer_clear(int W, int H, unsigned long long *zkey, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "zbuffer_clear", st);
    cudaMemsetAsync(zkey, 0, sizeof(unsigned long long) * (size_t)W * H, st);  // key 0: nothing splatted
}

size_t zsplat_defer_words(int V, int w, int h) {
    const size_t quads = (size_t)V * w * h;
    return kZdeferHead + std::max<size_t>(65536, quads / 64);
}

void launch_zbuffer_splat(int V, int w, int h, const float *depth, const WarpCams &cams, int W, int H,
                          unsigned long long *zkey, unsigned int *defer_q, cudaStream_t st, LaunchCounter &lc) {
    ProfScope _ps(lc, "zbuffer_splat", st);
    const int n = w * h;
    const int per_block = 256 * kZsplatPerThread;
    ZDefer defer{defer_q, defer_q ? (unsigned int)(zsplat_defer_words(V, w, h) - kZdeferHead) : 0u};
    if (defer_q) cudaMemsetAsync(defer_q, 0, sizeof(unsigned int), st);
    k_zsplat<<<dim3((n + per_block - 1) / per_block, V), 256, 0, st>>>(V, w, h, depth, cams, W, H, zkey, defer);
    lc.add(1);
    if (defer_q) {
        // one warp per queued quad, as many warps as two blocks per SM hold (the count is read on the device)
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        launch_pdl(k_zsplat_defer, dim3(2 * std::max(sms, 1)), dim3(256), 0, st, w, h, depth, cams, W, H, zkey, defer);
        lc.add(1);
    }
}

// ------------------------------------------------------------------ warps from depth maps without GL
// import_warps_from_depth (sources/import.cpp:243-450), float arithmetic as the reference's glm. WfdCams holds per
// camera (views, then the target at index V): fx, fy, cx, cy, row-major R, centre C, and P = K [R | t].
// Order-preserving uint key of a float (atomicMin on keys is min on floats, negative values included).
__device__ __forceinline__ unsigned int fkey(float f) {
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(unsigned int k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// X = d K^-1 (px, py, 1) with kc's K; world = R^T X + C with rc's R, C; out = P (world, 1) with pc's P.
__device__ __forceinline__ void wfd_transfer(const float *kc, const float *rc, const float *pc, float d, float px,
                                             float py, float out[3]) {
    // every product and sum rounded on its own (no FMA contraction), as the host arithmetic of the reference
    const float i00 = (float)(1.0 / (double)kc[0]), i11 = (float)(1.0 / (double)kc[1]);
    const float i20 = -__fdiv_rn(kc[2], kc[0]), i21 = -__fdiv_rn(kc[3], kc[1]);
    const float X0 = __fadd_rn(__fmul_rn(__fmul_rn(d, i00), px), __fmul_rn(d, i20));
    const float X1 = __fadd_rn(__fmul_rn(__fmul_rn(d, i11), py), __fmul_rn(d, i21));
    const float X2 = d;
    const float *R = rc + 4, *C = rc + 13;
    float Xw[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        Xw[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(R[0 * 3 + r], X0), __fmul_rn(R[1 * 3 + r], X1)),
                                    __fmul_rn(R[2 * 3 + r], X2)),
                          C[r]);
    const float *P = pc + 16;
#pragma unroll
    for (int r = 0; r < 3; ++r)
        out[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(P[r * 4 + 0], Xw[0]), __fmul_rn(P[r * 4 + 1], Xw[1])),
                                     __fmul_rn(P[r * 4 + 2], Xw[2])),
                           P[r * 4 + 3]);
}

__global__ void k_wfd_clear(size_t N, unsigned int *ukey) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) ukey[i] = fkey(1000.0f);
}

// Pass 1: warps and the target depth map (min over dsf x dsf pixels from int(tau) - dsf/2).
__global__ void k_wfd_project(int V, int w, int h, int dsf, const float *__restrict__ depth, int depth_channels,
                              const WfdCams cams, int W, int H, float *__restrict__ tau, unsigned int *ukey) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    const int n = w * h;
    if (m >= n) return;
    const float d = depth[(size_t)v * depth_channels * n + m];
    float *tv = tau + (size_t)v * 3 * n;
    if ((double)d < 1.0 / 1000.0 || 1000.0 < (double)d) {
        tv[m] = (float)-(double)w;
        tv[n + m] = tv[2 * n + m] = (float)-(double)h;
        return;
    }
    const float *c = cams.c[v], *u = cams.c[V];
    float X[3];
    wfd_transfer(c, c, u, d, (float)(m % w) + 0.5f, (float)(m / w) + 0.5f, X);
    const float txf = X[0] / X[2], tyf = X[1] / X[2];
    tv[m] = txf;
    tv[n + m] = tv[2 * n + m] = tyf;
    const unsigned int k = fkey(X[2]);
    for (int i = 0; i < dsf; ++i)
        for (int j = 0; j < dsf; ++j) {
            const int px = (int)txf - dsf / 2 + j, py = (int)tyf - dsf / 2 + i;
            if (0 <= px && px <= W - 1 && 0 <= py && py <= H - 1) atomicMin(ukey + (size_t)py * W + px, k);
        }
}

// Pass 2: coverage-weighted target depth over the footprint, back-projection, 10-pixel test.
__global__ void k_wfd_visibility(int V, int w, int h, int dsf, const WfdCams cams, int W, int H, int faithful,
                                 const unsigned int *__restrict__ ukey, float *__restrict__ tau) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    const int n = w * h;
    if (m >= n) return;
    float *tv = tau + (size_t)v * 3 * n;
    const double tx = tv[m], ty = tv[n + m];
    const double hd = (double)(float)dsf * 0.5;
    float u_d = 0.f, u_norm = 0.f;
    for (int i = 0; i < dsf + 1; ++i)
        for (int j = 0; j < dsf + 1; ++j) {
            const int px = (int)floor(tx - hd + 0.5) + j, py = (int)floor(ty - hd + 0.5) + i;
            if (!(0 <= px && px <= W - 1 && 0 <= py && py <= H - 1)) continue;
            const float zu = fkey_inv(ukey[(size_t)py * W + px]);
            if (zu == 1000.0f) continue;
            float dx = 1.0f, dy = 1.0f;
            if (j == 0) dx = (float)(((double)(float)px + 0.5) - (tx - hd));
            else if (j == dsf) dx = (float)((tx + hd) - ((double)(float)px - 0.5));
            if (i == 0) dy = (float)(((double)(float)py + 0.5) - (ty - hd));
            else if (i == dsf) dy = (float)((ty + hd) - ((double)(float)py - 0.5));
            u_d = __fadd_rn(u_d, __fmul_rn(__fmul_rn(dx, dy), zu));
            u_norm = __fadd_rn(u_norm, __fmul_rn(dx, dy));
        }
    if (u_norm == 0.0f) {
        tv[m] = (float)-(double)w;
        tv[n + m] = tv[2 * n + m] = (float)-(double)h;
        return;
    }
    u_d /= u_norm;
    const float *c = cams.c[v], *u = cams.c[V];
    float X[3];
    wfd_transfer(u, faithful ? c : u, c, u_d, (float)((int)tx) + 0.5f, (float)((int)ty) + 0.5f, X);
    const int ox = (int)(X[0] / X[2]), oy = (int)(X[1] / X[2]);
    const int x = m % w, y = m / w;
    if (ox - x < -10 || 10 < ox - x || oy - y < -10 || 10 < oy - y) {
        tv[m] = (float)(-(double)w * 2.0);
        tv[n + m] = tv[2 * n + m] = (float)(-(double)h * 2.0);
    }
}

void launch_warp_from_depth(int V, int w, int h, int dsf, const float *depth, int depth_channels, const WfdCams &cams,
                            int W, int H, int faithful, unsigned int *ukey, float *tau, cudaStream_t st,
                            LaunchCounter &lc) {
    ProfScope _ps(lc, "warp_from_depth", st);
    const size_t N = (size_t)W * H;
    const int n = w * h;
    k_wfd_clear<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, ukey);
    k_wfd_project<<<dim3((n + 255) / 256, V), 256, 0, st>>>(V, w, h, dsf, depth, depth_channels, cams, W, H, tau, ukey);
    k_wfd_visibility<<<dim3((n + 255) / 256, V), 256, 0, st>>>(V, w, h, dsf, cams, W, H, faithful, ukey, tau);
    lc.add(3);
}

// fromRadial2Ortho.frag:10-23: radial depth (and derivatives) to orthographic depth, in place. kinv holds K^-1
// (row-major) of each view; X = K^-1 (x + 1/2, y + 1/2, 1), d = |X|, z / d and the derivatives' chain rule.
__global__ void k_radial_to_ortho(int V, int w, int h, const WarpCams kinv, float *__restrict__ depth) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y;
    const int n = w * h;
    if (m >= n) return;
    const float *K = kinv.M[v];
    const float px = (m % w) + 0.5f, py = (m / w) + 0.5f;
    const float X0 = K[0] * px + K[1] * py + K[2], X1 = K[3] * px + K[4] * py + K[5], X2 = K[6] * px + K[7] * py + K[8];
    const float d = sqrtf(X0 * X0 + X1 * X1 + X2 * X2), d3 = d * d * d;
    const float c0 = X0 * K[0] + X1 * K[3] + X2 * K[6], c1 = X0 * K[1] + X1 * K[4] + X2 * K[7];
    float *dz = depth + (size_t)v * 3 * n;
    const float z = dz[m], zx = dz[n + m], zy = dz[2 * n + m];
    dz[m] = z / d;
    dz[n + m] = zx / d - z * c0 / d3;
    dz[2 * n + m] = zy / d - z * c1 / d3;
}

void launch_radial_to_ortho(int V, int w, int h, const WarpCams &kinv, float *depth, cudaStream_t st,
                            LaunchCounter &lc) {
    ProfScope _ps(lc, "radial_to_ortho", st);
    const int n = w * h;
    k_radial_to_ortho<<<dim3((n + 255) / 256, V), 256, 0, st>>>(V, w, h, kinv, depth);
    lc.add(1);
}

void launch_zbuffer_resolve(int W, int H, const unsigned long long *zkey, float *zbuf, cudaStream_t st,
                            LaunchCounter &lc) {
    ProfScope _ps(lc, "zbuffer_resolve", st);
    const size_t N = (size_t)W * H;
    k_zresolve<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, zkey, zbuf);
    lc.add(1);
}

void launch_tau(int V, int w, int h, const float *depth, const WarpCams &cams, int W, int H, const float *zbuf,
                float *tau3, float *dpart3, float *tau2, float *dp2, cudaStream_t st, LaunchCounter &lc,
                const BucketCount *bc, const unsigned long long *zkey) {
    ProfScope _ps(lc, "tau", st);
    const int n = w * h;
    const BucketCount count = bc ? *bc : BucketCount{};
    // programmatic launch: its launch overlaps the tail of the z-buffer kernel before it
    launch_pdl(k_tau, dim3((unsigned)((n + 256 * kTauPer - 1) / (256 * kTauPer)) * (unsigned)V), dim3(256), 0, st, V, w,
               h, depth, cams, W,
               H, zbuf, tau3, dpart3, tau2, dp2, count, zkey);
    lc.add(1);
}

}  // namespace lfrv
