// synth.cpp -- seeded synthetic light fields standing in for the reference's absent datasets.
//
// The reference's configs point at HCI / Strecha / Blender light fields under ./in/ that are not part of
// its repository. This generator produces scenes of the same shapes: an n x n grid of pinhole cameras
// (R = I, centres at baseline*(i-c, j-c, 0), t = -C, pinhole convention of sources/pinholeCamera.h:14-57),
// fronto-parallel textured planes, optional Gaussian depth bumps, per-view orthographic depth maps with
// analytic dz/dx, dz/dy (the (z, dz/dx, dz/dy) texture that depthSplatting.vert and tauWarp.frag read),
// inputs rendered at ss x resolution and box-decimated, and additive Gaussian sensor noise.
//
// The host form runs OpenMP over rows; the device form (lfrv_synth_scene_dev) runs the same tracing code, one
// thread per pixel. The arithmetic is plain IEEE double with a portable polynomial sine so that x86-64 and
// aarch64 hosts produce the same scenes (host code built with -ffp-contract=off, device code with -fmad=false).
// The device form multiplies by reciprocals where the host form divides (sine reduction, bump falloff), and its
// double exp, log and cos may differ from the host library's in the last bit, so the two forms agree to the
// rounding of the final float in all but rare pixels.
#include "context.h"
#include "lfrv.h"
#include "lfrv_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#define LFRV_HD __host__ __device__ __forceinline__

namespace {

// ------------------------------------------------------------------ Philox4x32-10 (Salmon et al. 2011)
struct Philox {
    static LFRV_HD void round(uint32_t ctr[4], const uint32_t key[2]) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t out[4] = {hi1 ^ ctr[1] ^ key[0], lo1, hi0 ^ ctr[3] ^ key[1], lo0};
        for (int i = 0; i < 4; ++i) ctr[i] = out[i];
    }
    static LFRV_HD void gen(uint64_t seed, uint64_t c0, uint64_t c1, uint32_t out[4]) {
        uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
        uint32_t ctr[4] = {(uint32_t)c0, (uint32_t)(c0 >> 32), (uint32_t)c1, (uint32_t)(c1 >> 32)};
        for (int r = 0; r < 10; ++r) {
            round(ctr, key);
            key[0] += 0x9E3779B9u;
            key[1] += 0xBB67AE85u;
        }
        for (int i = 0; i < 4; ++i) out[i] = ctr[i];
    }
};

LFRV_HD double u01(uint32_t a, uint32_t b) {  // 53-bit uniform in (0,1)
    const uint64_t v = ((uint64_t)a << 21) ^ (uint64_t)b;
    return ((double)(v & ((1ull << 53) - 1)) + 0.5) * (1.0 / 9007199254740992.0);
}

// Sequential seeded stream for scene layout (planes, frequencies, bumps).
struct Stream {
    uint64_t seed, n = 0;
    explicit Stream(uint64_t s) : seed(s) {}
    double uniform() {
        uint32_t o[4];
        Philox::gen(seed, n++, 0x5ce7e, o);
        return u01(o[0], o[1]);
    }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

// Portable sine: reduction to [-pi/2, pi/2] and a degree-19 Taylor polynomial (error < 3e-14).
LFRV_HD double psin(double x) {
    const double twopi = 6.283185307179586476925286766559;
    const double pi = 3.1415926535897932384626433832795;
#ifdef __CUDA_ARCH__
    x -= twopi * nearbyint(x * (1.0 / twopi));  // a multiple of 2 pi off only at a half-period, where it is harmless
#else
    x -= twopi * nearbyint(x / twopi);
#endif
    if (x > 0.5 * pi) x = pi - x;
    else if (x < -0.5 * pi) x = -pi - x;
    const double x2 = x * x;
    double p = -1.0 / 121645100408832000.0;  // -1/19!
    p = p * x2 + 1.0 / 355687428096000.0;    // 1/17!
    p = p * x2 - 1.0 / 1307674368000.0;      // 1/15!
    p = p * x2 + 1.0 / 6227020800.0;         // 1/13!
    p = p * x2 - 1.0 / 39916800.0;           // 1/11!
    p = p * x2 + 1.0 / 362880.0;             // 1/9!
    p = p * x2 - 1.0 / 5040.0;               // 1/7!
    p = p * x2 + 1.0 / 120.0;                // 1/5!
    p = p * x2 - 1.0 / 6.0;                  // 1/3!
    p = p * x2 + 1.0;
    return x * p;
}

constexpr int kSines = 64;

struct Plane {
    double depth;
    double x0, x1, y0, y1;  // world rectangle; ignored for the background
    bool full;
    double a[3][kSines], b[3][kSines], phi[3][kSines];  // phase = a*X + b*Y + phi
};

struct Bump {
    int plane;
    double X, Y, amp, sig;
    double inv_s2;  // 1 / sig^2 (the device form multiplies by it where the host form divides)
};

struct Scene {
    std::vector<Plane> planes;  // ascending depth
    std::vector<Bump> bumps;
};

// What the tracer reads: the planes and bumps as arrays (host vectors, or a copy in device memory).
struct SceneView {
    const Plane *planes;
    int nplanes;
    const Bump *bumps;
    int nbumps;
};
inline SceneView view_of(const Scene &s) {
    return SceneView{s.planes.data(), (int)s.planes.size(), s.bumps.data(), (int)s.bumps.size()};
}

struct Hit {
    double z, zx, zy;  // depth and derivatives wrt the rendering camera's pixel coordinates
    double col[3];
};

Scene make_scene(const lfrv_scene_params &p, double world_width_per_depth) {
    Scene s;
    Stream rng(p.seed * 0x9E3779B97F4A7C15ull + 0x1234567ull);
    for (int k = 0; k < p.nplanes; ++k) {
        Plane pl;
        pl.depth = p.depths[k];
        pl.full = (k == p.nplanes - 1);
        // Rectangle inside the target's field of view at this depth.
        const double half = 0.5 * world_width_per_depth * pl.depth;
        const double wx = rng.uniform(0.3, 0.7) * 2.0 * half, wy = rng.uniform(0.3, 0.7) * 2.0 * half;
        const double cx = rng.uniform(-0.5, 0.5) * half, cy = rng.uniform(-0.5, 0.5) * half;
        pl.x0 = cx - 0.5 * wx;
        pl.x1 = cx + 0.5 * wx;
        pl.y0 = cy - 0.5 * wy;
        pl.y1 = cy + 0.5 * wy;
        // Texture: cycles per target image width at the plane's depth.
        const double ww = world_width_per_depth * pl.depth;
        for (int c = 0; c < 3; ++c)
            for (int j = 0; j < kSines; ++j) {
                const double f = rng.uniform(0.5, 40.0);
                const double ang = rng.uniform(0.0, 6.283185307179586);
                pl.a[c][j] = 6.283185307179586 * f * std::cos(ang) / ww;
                pl.b[c][j] = 6.283185307179586 * f * std::sin(ang) / ww;
                pl.phi[c][j] = rng.uniform(0.0, 6.283185307179586);
            }
        s.planes.push_back(pl);
    }
    for (int i = 0; i < p.nbumps; ++i) {
        Bump b;
        b.plane = (int)std::min<double>(p.nplanes - 1, std::floor(rng.uniform() * p.nplanes));
        const Plane &pl = s.planes[b.plane];
        const double half = 0.5 * world_width_per_depth * pl.depth;
        if (pl.full) {
            b.X = rng.uniform(-half, half);
            b.Y = rng.uniform(-half, half);
        } else {
            b.X = rng.uniform(pl.x0, pl.x1);
            b.Y = rng.uniform(pl.y0, pl.y1);
        }
        b.amp = (rng.uniform() < 0.5 ? -1.0 : 1.0) * p.bump_amp;
        // sigma in target pixels -> world units at the plane's depth
        b.sig = p.bump_sigma_px * world_width_per_depth * pl.depth / (double)(p.w * p.dsf);
        b.inv_s2 = 1.0 / (b.sig * b.sig);
        s.bumps.push_back(b);
    }
    return s;
}

// Height field of plane k: depth(X,Y) and its gradient.
LFRV_HD void height(const SceneView &s, int k, double X, double Y, double &h, double &hX, double &hY) {
    h = s.planes[k].depth;
    hX = hY = 0.0;
    for (int i = 0; i < s.nbumps; ++i) {
        const Bump &b = s.bumps[i];
        if (b.plane != k) continue;
        const double dx = X - b.X, dy = Y - b.Y;
#ifdef __CUDA_ARCH__
        // FP64 division is a long sequence on this GPU's narrow FP64 pipe: multiply by the reciprocal
        const double r2 = (dx * dx + dy * dy) * b.inv_s2;
        if (r2 > 64.0) continue;
        const double e = b.amp * exp(-0.5 * r2);
        h += e;
        hX -= e * dx * b.inv_s2;
        hY -= e * dy * b.inv_s2;
#else
        const double r2 = (dx * dx + dy * dy) / (b.sig * b.sig);
        if (r2 > 64.0) continue;
        const double e = b.amp * exp(-0.5 * r2);
        h += e;
        hX -= e * dx / (b.sig * b.sig);
        hY -= e * dy / (b.sig * b.sig);
#endif
    }
}

// Nearest surface hit of the ray through pixel-space point (px,py) of a camera at centre (Cx,Cy,0)
// with focal f and principal point (cx,cy), R = I.
LFRV_HD bool trace(const SceneView &s, double Cx, double Cy, double f, double cx, double cy, double px, double py,
                   bool want_colour, Hit &hit) {
    const double u = (px - cx) / f, v = (py - cy) / f;
    for (int k = 0; k < s.nplanes; ++k) {
        const Plane &pl = s.planes[k];
        double Z = pl.depth, h, hX, hY;
        // Newton on g(Z) = Z - h(Cx + Z u, Cy + Z v)
        for (int it = 0; it < 16; ++it) {
            height(s, k, Cx + Z * u, Cy + Z * v, h, hX, hY);
            const double g = Z - h;
            double gp = 1.0 - (hX * u + hY * v);
            if (fabs(gp) < 0.2) gp = gp < 0 ? -0.2 : 0.2;
            const double step = g / gp;
            Z -= step;
            if (fabs(step) < 1e-13) break;
        }
        height(s, k, Cx + Z * u, Cy + Z * v, h, hX, hY);
        const double X = Cx + Z * u, Y = Cy + Z * v;
        if (!pl.full && (X < pl.x0 || X > pl.x1 || Y < pl.y0 || Y > pl.y1)) continue;
        hit.z = Z;
        const double den = 1.0 - hX * u - hY * v;
        hit.zx = hX * Z / f / den;
        hit.zy = hY * Z / f / den;
        if (want_colour) {
            for (int c = 0; c < 3; ++c) {
                double acc = 0.0;
                for (int j = 0; j < kSines; ++j) acc += psin(pl.a[c][j] * X + pl.b[c][j] * Y + pl.phi[c][j]);
                hit.col[c] = 0.5 + (0.5 / kSines) * acc;
            }
        }
        return true;
    }
    return false;
}

LFRV_HD double gauss(uint64_t seed, uint64_t view, uint64_t idx) {
    uint32_t o[4];
    Philox::gen(seed ^ 0xA5A5A5A5DEADBEEFull, view, idx, o);
    const double u1 = u01(o[0], o[1]), u2 = u01(o[2], o[3]);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// One input pixel of a view: the ss x ss samples' colours averaged, plus noise (as lfrv_synth_scene's loop).
LFRV_HD void view_pixel(const SceneView &s, const lfrv_scene_params &p, int v, double Cx, double Cy, double fr,
                        double cxr, double cyr, int x, int y, int w, size_t plane_in, float *out) {
    const int ss = p.ss;
    Hit hit;
    double acc[3] = {0, 0, 0};
    for (int sy = 0; sy < ss; ++sy)
        for (int sx = 0; sx < ss; ++sx) {
            const double px = x * ss + sx + 0.5, py = y * ss + sy + 0.5;
            if (trace(s, Cx, Cy, fr, cxr, cyr, px, py, true, hit))
                for (int ch = 0; ch < 3; ++ch) acc[ch] += hit.col[ch];
        }
    const size_t o = (size_t)y * w + x;
    for (int ch = 0; ch < 3; ++ch) {
        double val = acc[ch] / (ss * ss);
        if (p.noise_sigma > 0) val += p.noise_sigma * gauss(p.seed, (uint64_t)v, (uint64_t)(ch * plane_in + o));
        out[ch * plane_in + o] = (float)val;
    }
}

// One input pixel's depth map entry (z, dz/dx, dz/dy), or INVALID_DEPTH where the ray hits nothing
// (sources/openGL/frameBuffer.h:13).
LFRV_HD void depth_pixel(const SceneView &s, double Cx, double Cy, double f, int x, int y, int w, int h,
                         size_t plane_in, float *out) {
    Hit hit;
    const size_t o = (size_t)y * w + x;
    if (trace(s, Cx, Cy, f, 0.5 * w, 0.5 * h, x + 0.5, y + 0.5, false, hit)) {
        out[o] = (float)hit.z;
        out[plane_in + o] = (float)hit.zx;
        out[2 * plane_in + o] = (float)hit.zy;
    } else {
        out[o] = 1000.0f;
        out[plane_in + o] = 0.0f;
        out[2 * plane_in + o] = 0.0f;
    }
}

LFRV_HD void gt_pixel(const SceneView &s, double f, int x, int y, int W, int H, float *gt) {
    Hit hit;
    const size_t o = (size_t)y * W + x, plane_out = (size_t)W * H;
    const bool ok = trace(s, 0.0, 0.0, f, 0.5 * W, 0.5 * H, x + 0.5, y + 0.5, true, hit);
    for (int ch = 0; ch < 3; ++ch) gt[ch * plane_out + o] = ok ? (float)hit.col[ch] : 0.0f;
}

// ------------------------------------------------------------------ device form
// Camera centres of the input views (views in lfrv_synth_scene's order), passed by value.
struct SynthCentres {
    double C[2 * 255];
};

__global__ void k_synth_views(SceneView s, lfrv_scene_params p, SynthCentres cs, double fr, double cxr, double cyr,
                              float *views) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, v = blockIdx.z;
    if (x >= p.w || y >= p.h) return;
    const size_t plane_in = (size_t)p.w * p.h;
    view_pixel(s, p, v, cs.C[2 * v], cs.C[2 * v + 1], fr, cxr, cyr, x, y, p.w, plane_in,
               views + (size_t)v * 3 * plane_in);
}

__global__ void k_synth_depth(SceneView s, lfrv_scene_params p, SynthCentres cs, double f, float *depth) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, v = blockIdx.z;
    if (x >= p.w || y >= p.h) return;
    const size_t plane_in = (size_t)p.w * p.h;
    depth_pixel(s, cs.C[2 * v], cs.C[2 * v + 1], f, x, y, p.w, p.h, plane_in, depth + (size_t)v * 3 * plane_in);
}

__global__ void k_synth_gt(SceneView s, double f, int W, int H, float *gt) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    gt_pixel(s, f, x, y, W, H, gt);
}

void camera(lfrv_camera &c, double f, int W, int H, double Cx, double Cy) {
    std::memset(&c, 0, sizeof(c));
    c.K[0] = (float)f;
    c.K[2] = (float)(0.5 * W);
    c.K[4] = (float)f;
    c.K[5] = (float)(0.5 * H);
    c.K[8] = 1.0f;
    c.R[0] = c.R[4] = c.R[8] = 1.0f;
    c.t[0] = (float)(-Cx);
    c.t[1] = (float)(-Cy);
    c.t[2] = 0.0f;
    c.width = W;
    c.height = H;
}

}  // namespace

extern "C" int lfrv_scene_params_preset(int which, lfrv_scene_params *p) {
    if (!p) return lfrv::fail(LFRV_E_ARG, "null params");
    std::memset(p, 0, sizeof(*p));
    p->focal_per_256 = 300.0;
    p->seed = 1;
    if (which == 1) {
        p->grid = 3;
        p->w = p->h = 256;
        p->ss = 1;
        p->dsf = 1;
        p->baseline = 0.05;
        p->nplanes = 3;
        p->depths[0] = 1.0;
        p->depths[1] = 1.5;
        p->depths[2] = 2.5;
        p->noise_sigma = 0.01;
    } else if (which == 2) {
        p->grid = 5;
        p->w = p->h = 512;
        p->ss = 2;
        p->dsf = 2;
        p->baseline = 0.03;
        p->nplanes = 5;
        const double d[5] = {1.0, 1.3, 1.7, 2.2, 3.0};
        for (int i = 0; i < 5; ++i) p->depths[i] = d[i];
        p->nbumps = 20;
        p->bump_amp = 0.1;
        p->bump_sigma_px = 30.0;
        p->noise_sigma = 0.005;
    } else {
        return lfrv::fail(LFRV_E_ARG, "unknown scene preset %d", which);
    }
    return LFRV_OK;
}

extern "C" int lfrv_synth_scene(const lfrv_scene_params *p, float *views, float *depth, lfrv_camera *cams,
                                float *gt) {
    if (!p || p->grid < 2 || p->w <= 0 || p->h <= 0 || p->ss < 1 || p->dsf < 1 || p->nplanes < 1 ||
        p->nplanes > 16)
        return lfrv::fail(LFRV_E_ARG, "bad scene parameters");
    const int n = p->grid, w = p->w, h = p->h, W = w * p->dsf, H = h * p->dsf;
    const int center = (n / 2) * n + (n / 2);
    const double c = 0.5 * (n - 1);
    const double f_target = p->focal_per_256 * (double)W / 256.0;
    const double f_input = f_target / p->dsf;
    const double world_width_per_depth = (double)W / f_target;
    const Scene scene = make_scene(*p, world_width_per_depth);
    const SceneView sv = view_of(scene);
    const size_t plane_in = (size_t)w * h;

    int v = 0;
    for (int s = 0; s < n * n; ++s) {
        if (s == center) continue;
        const int i = s % n, j = s / n;
        const double Cx = p->baseline * (i - c), Cy = p->baseline * (j - c);
        if (cams) camera(cams[v], f_input, w, h, Cx, Cy);
        if (views) {
            const int ss = p->ss;
            const double fr = f_input * ss, cxr = 0.5 * w * ss, cyr = 0.5 * h * ss;
            float *out = views + (size_t)v * 3 * plane_in;
#pragma omp parallel for schedule(dynamic, 4)
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x) view_pixel(sv, *p, v, Cx, Cy, fr, cxr, cyr, x, y, w, plane_in, out);
        }
        if (depth) {
            float *out = depth + (size_t)v * 3 * plane_in;
#pragma omp parallel for schedule(dynamic, 4)
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x) depth_pixel(sv, Cx, Cy, f_input, x, y, w, h, plane_in, out);
        }
        ++v;
    }
    if (cams) camera(cams[v], f_target, W, H, 0.0, 0.0);
    if (gt) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) gt_pixel(sv, f_target, x, y, W, H, gt);
    }
    return LFRV_OK;
}

extern "C" int lfrv_synth_scene_dev(lfrv_ctx *ctx, const lfrv_scene_params *p, float *d_views, float *d_depth,
                                    lfrv_camera *cams, float *d_gt) {
    LFRV_API_BEGIN
    if (!ctx) return lfrv::fail(LFRV_E_ARG, "null context");
    LFRV_CUDA(cudaSetDevice(ctx->device));
    if (!p || p->grid < 2 || p->w <= 0 || p->h <= 0 || p->ss < 1 || p->dsf < 1 || p->nplanes < 1 ||
        p->nplanes > 16 || p->grid * p->grid - 1 > 255 || p->nbumps < 0)
        lfrv::raise(LFRV_E_ARG, "bad scene parameters");
    const int n = p->grid, w = p->w, h = p->h, W = w * p->dsf, H = h * p->dsf;
    const int center = (n / 2) * n + (n / 2);
    const double c = 0.5 * (n - 1);
    const double f_target = p->focal_per_256 * (double)W / 256.0;
    const double f_input = f_target / p->dsf;
    const Scene scene = make_scene(*p, (double)W / f_target);
    // the planes and bumps in device memory (the context's scene buffer)
    const size_t pb = sizeof(Plane) * scene.planes.size(), bb = sizeof(Bump) * scene.bumps.size();
    lfrv::Workspace &ws = ctx->ws;
    ws.scene.ensure(pb + bb + 16);
    char *dscene = ws.scene.as<char>();
    LFRV_CUDA(cudaMemcpyAsync(dscene, scene.planes.data(), pb, cudaMemcpyHostToDevice, ctx->stream));
    if (bb) LFRV_CUDA(cudaMemcpyAsync(dscene + pb, scene.bumps.data(), bb, cudaMemcpyHostToDevice, ctx->stream));
    const SceneView sv{reinterpret_cast<const Plane *>(dscene), (int)scene.planes.size(),
                       reinterpret_cast<const Bump *>(dscene + pb), (int)scene.bumps.size()};
    SynthCentres cs;
    std::memset(&cs, 0, sizeof(cs));
    int v = 0;
    for (int s = 0; s < n * n; ++s) {
        if (s == center) continue;
        const double Cx = p->baseline * (s % n - c), Cy = p->baseline * (s / n - c);
        cs.C[2 * v] = Cx;
        cs.C[2 * v + 1] = Cy;
        if (cams) camera(cams[v], f_input, w, h, Cx, Cy);
        ++v;
    }
    if (cams) camera(cams[v], f_target, W, H, 0.0, 0.0);
    const dim3 b(16, 8);
    const dim3 gi((w + 15) / 16, (h + 7) / 8, v);
    if (d_views)
        k_synth_views<<<gi, b, 0, ctx->stream>>>(sv, *p, cs, f_input * p->ss, 0.5 * w * p->ss, 0.5 * h * p->ss,
                                                 d_views);
    if (d_depth) k_synth_depth<<<gi, b, 0, ctx->stream>>>(sv, *p, cs, f_input, d_depth);
    if (d_gt) k_synth_gt<<<dim3((W + 15) / 16, (H + 7) / 8), b, 0, ctx->stream>>>(sv, f_target, W, H, d_gt);
    ctx->launches.add((d_views ? 1 : 0) + (d_depth ? 1 : 0) + (d_gt ? 1 : 0));
    LFRV_CUDA(cudaGetLastError());
    // the scene buffer is reused by the next call: the host's copies above must be done with their sources
    LFRV_CUDA(cudaStreamSynchronize(ctx->stream));
    LFRV_API_END
}

extern "C" double lfrv_psnr(int W, int H, const float *a, const float *b, int border) {
    if (!a || !b || W <= 2 * border || H <= 2 * border) return -1.0;
    double mse_t = 0.0;
    for (int ch = 0; ch < 3; ++ch) {
        double mse = 0.0;
        for (int y = border; y < H - border; ++y)
            for (int x = border; x < W - border; ++x) {
                const size_t o = (size_t)ch * W * H + (size_t)y * W + x;
                const double d = (double)a[o] - (double)b[o];
                mse += d * d;
            }
        mse_t += mse / ((double)(W - 2 * border) * (H - 2 * border));
    }
    mse_t /= 3.0;
    if (mse_t == 0.0) return 1e300;
    return 10.0 * std::log10(1.0 / mse_t);
}
