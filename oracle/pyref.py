"""ctypes binding of oracle/_ref/libref_kernels.so: the reference's own kernels compiled for the CPU.

TEST INFRASTRUCTURE (built by oracle/build_ref.sh where the reference tree exists). The helpers below
compose the kernels in the order the reference's host code launches them, so the oracle's stage functions
can be compared with the reference's arithmetic bit for bit.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_ref" / "libref_kernels.so"
LIB = C.CDLL(str(LIB_PATH)) if LIB_PATH.exists() else None

_f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
_u8 = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint8))  # noqa: E731
_i = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
F = C.c_float


def available() -> bool:
    return LIB is not None


def cells(tx: np.ndarray, ty: np.ndarray, W: int, H: int) -> np.ndarray:
    """Source pixels vtv_sr_init_forward_warp_structure_unstructured puts into cells (optimization.cu:906-927),
    in index order (one segment)."""
    tx = tx.ravel().astype(np.float32)
    ty = ty.ravel().astype(np.float32)
    out = ~((tx < 0) | (ty < 0) | (tx > W) | (ty > H))
    px = np.floor((tx.astype(np.float64) - 0.5).astype(np.float32)).astype(np.int64)
    py = np.floor((ty.astype(np.float64) - 0.5).astype(np.float32)).astype(np.int64)
    ok = out & (px >= 0) & (py >= 0) & (px <= W - 1) & (py <= H - 1)
    return np.ascontiguousarray(np.nonzero(ok)[0].astype(np.int32))


class View:
    def __init__(self, img, tx, ty, W, H, dsf):
        self.img = np.ascontiguousarray(img, np.float32)
        self.tx = np.ascontiguousarray(tx, np.float32).ravel().copy()
        self.ty = np.ascontiguousarray(ty, np.float32).ravel().copy()
        self.h, self.w = tx.shape
        self.W, self.H, self.dsf, self.ks = W, H, dsf, dsf + 1
        self.A = np.zeros(self.h * self.w * self.ks * self.ks, np.float32)
        LIB.ref_set_A_bilinear(W, H, self.w, self.h, self.ks, _f(self.tx), _f(self.ty), _f(self.A))
        self.cells = cells(self.tx, self.ty, W, H)

    def gather3(self, U):
        n = self.w * self.h
        o = np.zeros((3, n), np.float32)
        U = np.ascontiguousarray(U, np.float32)
        N = self.W * self.H
        Uf = U.reshape(3, N)
        LIB.ref_convolution_rgb(self.W, self.H, self.w, self.h, self.ks, _f(self.A), _f(self.tx), _f(self.ty),
                                _f(Uf[0]), _f(Uf[1]), _f(Uf[2]), _f(o[0]), _f(o[1]), _f(o[2]))
        return o

    def gather1(self, X):
        o = np.zeros(self.w * self.h, np.float32)
        X = np.ascontiguousarray(X, np.float32).ravel()
        LIB.ref_convolution_1(self.W, self.H, self.w, self.h, self.ks, _f(self.A), _f(self.tx), _f(self.ty), _f(X),
                              _f(o))
        return o

    def splat3(self, src3, out3, norm, use_A=True):
        LIB.ref_deconvolution_rgb(self.W, self.H, _f(src3[0]), _f(src3[1]), _f(src3[2]), _i(self.cells), 0,
                                  len(self.cells), self.ks, self.dsf, _f(self.A) if use_A else None, _f(self.tx),
                                  _f(self.ty), _f(out3[0]), _f(out3[1]), _f(out3[2]), _f(norm))

    def splat1(self, src, out, norm):
        LIB.ref_deconvolution_1(self.W, self.H, _f(src), _i(self.cells), 0, len(self.cells), self.ks, self.dsf,
                                _f(self.A), _f(self.tx), _f(self.ty), _f(out), _f(norm))

    def weighted_splat(self, wgt, out3, norm):
        img = self.img.reshape(3, -1)
        LIB.ref_weighted_deconvolution(self.W, self.H, _f(img[0]), _f(img[1]), _f(img[2]), _i(self.cells), 0,
                                       len(self.cells), self.ks, self.dsf, _f(self.A), _f(wgt), _f(self.tx),
                                       _f(self.ty), _f(out3[0]), _f(out3[1]), _f(out3[2]), _f(norm))


def views_of(views, tau, w, h, dsf):
    W, H = w * dsf, h * dsf
    return [View(views[v], tau[v, 0], tau[v, 1], W, H, dsf) for v in range(views.shape[0])]


# ---------------------------------------------------------------- compositions of the reference's launches
def visibility(tau, w, h, dsf):
    """coco_vtv_setup_visibility_mask (sources/optimization.cu:33-135)."""
    W, H = w * dsf, h * dsf
    vs = views_of(np.zeros((tau.shape[0], 3, h, w), np.float32), tau, w, h, dsf)
    ones = np.ones(W * H, np.float32)
    cov = np.zeros(W * H, np.float32)
    norm = np.zeros(W * H, np.float32)
    for v in vs:
        v.splat1(ones, cov, norm)
    vis = np.zeros(W * H, np.uint8)
    LIB.ref_visibility_threshold(W, H, _f(cov), _u8(vis))
    return cov.reshape(H, W), vis.reshape(H, W)


def weights(views, tau, dpart, U, vis, gx0, gy0, w, h, dsf, sigma, thr):
    """coco_vtv_sr_compute_weights_unstructured (sources/optimization.cu:1066-1167) with explicit gradient
    buffers (their prior content survives where the masked Sobel does not write)."""
    W, H = w * dsf, h * dsf
    n = w * h
    U = np.ascontiguousarray(U, np.float32)
    gx, gy = np.array(gx0, np.float32), np.array(gy0, np.float32)
    LIB.ref_compute_gradient(W, H, _f(U[0]), _f(U[1]), _f(U[2]), _f(gx), _f(gy), _u8(np.ascontiguousarray(vis)))
    out = np.zeros((views.shape[0], n), np.float32)
    for k, v in enumerate(views_of(views, tau, w, h, dsf)):
        ax, ay = v.gather1(gx), v.gather1(gy)
        dpx = (dpart[k, 1].ravel() * dpart[k, 0].ravel()).astype(np.float32)  # sigma_z * dtau/dz
        dpy = (dpart[k, 2].ravel() * dpart[k, 0].ravel()).astype(np.float32)
        ang = np.zeros(n, np.float32)
        LIB.ref_angular_weights(w, h, _f(ax), _f(ay), sigma, _f(dpx), _f(dpy), thr, _f(ang))
        dfm = np.zeros(n, np.float32)
        LIB.ref_gold_deform_weights(W, H, w, h, _f(v.tx), _f(v.ty), _f(dfm))
        LIB.ref_multiply_with(w, h, _f(ang), _f(dfm))
        out[k] = ang
    return gx, gy, out.reshape(views.shape[0], h, w)


def laplacian(X, W, H):
    """cuda_laplacian_device (vtv_sr_kernels_unstructured.cu:720-760) without a visibility mask."""
    X = np.ascontiguousarray(X, np.float32).ravel()
    out = np.zeros(W * H, np.float32)
    LIB.ref_laplacian(W, H, _f(X), _f(out))
    return out


def dataterm(views, tau, wg, U, w, h, dsf, sigma, alpha, lam, beta=0.0, gw_type=0, gradient_step=0.1):
    """vtv_sr_dataterm_intensities (optimization.cu:1835-1966), vtv_sr_dataterm_gradients (:1969-2116) when
    beta > 0, and F of vtv_sr_ista_step_unstructured (:1775-1812). Returns G (before the [-1,1] clamp) and F."""
    W, H = w * dsf, h * dsf
    N, n = W * H, w * h
    wg = np.ascontiguousarray(wg, np.float32).reshape(-1, n)
    vlist = views_of(views, tau, w, h, dsf)
    G = np.zeros((3, N), np.float32)
    s2 = np.float32(sigma) * np.float32(sigma)
    if alpha > 0:
        Gi = np.zeros((3, N), np.float32)
        norm = np.zeros(N, np.float32)
        for k, v in enumerate(vlist):
            t = v.gather3(U)
            img = v.img.reshape(3, n)
            for c in range(3):
                LIB.ref_subtract_from(w, h, _f(img[c]), _f(t[c]))
            for c in range(3):
                LIB.ref_multiply_with(w, h, _f(t[c]), _f(wg[k]))
            v.splat3(t, Gi, norm)
        for c in range(3):
            LIB.ref_normalize(W, H, _f(Gi[c]), _f(norm))
            LIB.ref_scale(W, H, _f(Gi[c]), s2)
            LIB.ref_add_scaled_to(W, H, _f(Gi[c]), alpha, _f(G[c]))
    if beta > 0:
        Gg = np.zeros((3, N), np.float32)
        norm = np.zeros(N, np.float32)
        Uf = np.ascontiguousarray(U, np.float32).reshape(3, N)
        for k, v in enumerate(vlist):
            lu = np.stack([laplacian(Uf[c], W, H) for c in range(3)])
            t = v.gather3(lu)
            img = v.img.reshape(3, n)
            for c in range(3):
                LIB.ref_scale(w, h, _f(t[c]), float(dsf * dsf))
                lv = laplacian(img[c], w, h)
                LIB.ref_subtract_from(w, h, _f(lv), _f(t[c]))
            if gw_type != 0:
                for c in range(3):
                    LIB.ref_multiply_with(w, h, _f(t[c]), _f(wg[k]))
            v.splat3(t, Gg, norm)
        for c in range(3):
            LIB.ref_normalize(W, H, _f(Gg[c]), _f(norm))
            if gw_type != 0:
                LIB.ref_scale(W, H, _f(Gg[c]), s2)
            LIB.ref_scale(W, H, _f(Gg[c]), -np.float32(gradient_step))
            LIB.ref_add_scaled_to(W, H, _f(Gg[c]), beta, _f(G[c]))
    Gout = G.copy()
    L = np.float32(1.0 / np.float64(np.float32(lam)))
    fscale = np.float32(-1.0 / np.float64(np.float32(lam) * L))
    Uq = np.ascontiguousarray(U, np.float32).reshape(3, N).copy()
    for c in range(3):
        LIB.ref_clamp(W, H, _f(G[c]), -1.0, 1.0)
        LIB.ref_scale(W, H, _f(G[c]), fscale)
        LIB.ref_add_to(W, H, _f(Uq[c]), _f(G[c]))
        LIB.ref_clamp(W, H, _f(G[c]), 0.0, 1.0)
    return Gout.reshape(3, H, W), G.reshape(3, H, W)


def rof(niter, tau, sigma, lam, F, g, U, P):
    """niter inner iterations as vtv_sr_ista_step_unstructured launches them (optimization.cu:1815-1828)."""
    F = np.ascontiguousarray(F, np.float32)
    g = np.ascontiguousarray(g, np.float32)
    u, pp = np.array(U, np.float32), np.array(P, np.float32)
    H, W = u.shape[1], u.shape[2]
    for _ in range(niter):
        for c in range(3):
            LIB.ref_rof_dual_step(W, H, sigma, _f(u[c]), _f(pp[2 * c]), _f(pp[2 * c + 1]))
        LIB.ref_reproject_tvf_weighted(W, H, _f(g), *[_f(pp[k]) for k in range(6)])
        for c in range(3):
            LIB.ref_primal_prox(W, H, tau, lam, _f(u[c]), _f(u[c]), _f(F[c]), _f(pp[2 * c]), _f(pp[2 * c + 1]))
    return u, pp


def initial_image(views, tau, wg, w, h, dsf):
    """Weighted splat + normalise of coco_vtv_sr_compute_initial_image (optimization.cu:1300-1344)."""
    W, H = w * dsf, h * dsf
    N, n = W * H, w * h
    wg = np.ascontiguousarray(wg, np.float32).reshape(-1, n)
    U = np.zeros((3, N), np.float32)
    norm = np.zeros(N, np.float32)
    for k, v in enumerate(views_of(views, tau, w, h, dsf)):
        v.weighted_splat(wg[k], U, norm)
    for c in range(3):
        LIB.ref_normalize(W, H, _f(U[c]), _f(norm))
    return U.reshape(3, H, W), norm.reshape(H, W)


def regularizer_g0(tau, wg, norm_prior, w, h, dsf, sigma, lam, lmf):
    """coco_vtv_sr_init_regularizer_weight_unstructured (optimization.cu:2251-2319) up to the blur."""
    W, H = w * dsf, h * dsf
    N, n = W * H, w * h
    wg = np.ascontiguousarray(wg, np.float32).reshape(-1, n)
    vs = views_of(np.zeros((tau.shape[0], 3, h, w), np.float32), tau, w, h, dsf)
    m = np.zeros(N, np.float32)
    nm = np.zeros(N, np.float32) if norm_prior is None else np.array(norm_prior, np.float32).ravel().copy()
    for k, v in enumerate(vs):
        v.splat1(wg[k], m, nm)
    LIB.ref_normalize(W, H, _f(m), _f(nm))
    LIB.ref_scale(W, H, _f(m), np.float32(sigma) * np.float32(sigma))
    g0 = np.zeros(N, np.float32)
    lmax = np.float32(lmf) * np.float32(lam)
    LIB.ref_regularizer_weight(W, H, lmax, lam, float(len(vs)), _f(m), _f(g0))
    return nm.reshape(H, W), g0.reshape(H, W)


def push_pull(U, vis):
    """coco_vtv_push_pull (optimization.cu:544-651) with the reference's reduce / expand; U = filled - U."""
    U = np.ascontiguousarray(U, np.float32)
    H, W = U.shape[1], U.shape[2]
    out = np.zeros_like(U)
    for c in range(3):
        img = [U[c].ravel().copy()]
        vp = [np.ascontiguousarray(vis, np.uint8).ravel().copy()]
        for s in range(1, 11):
            Ws, Hs, ws, hs = W >> (s - 1), H >> (s - 1), W >> s, H >> s
            img.append(np.zeros(max(ws * hs, 1), np.float32))
            vp.append(np.zeros(max(ws * hs, 1), np.uint8))
            if ws > 0 and hs > 0:
                LIB.refp_reduce(Ws, Hs, ws, hs, _f(img[s - 1]), _f(img[s]))
                LIB.refp_reduce_bool(Ws, Hs, ws, hs, _u8(vp[s - 1]), _u8(vp[s]))
        for s in range(10, 0, -1):
            Ws, Hs, ws, hs = W >> (s - 1), H >> (s - 1), W >> s, H >> s
            if Ws > 0 and Hs > 0 and ws > 0 and hs > 0:
                LIB.refp_expand(Ws, Hs, ws, hs, _f(img[s]), _f(img[s - 1]), _u8(vp[s - 1]))
        out[c] = img[0].reshape(H, W) - U[c]
    return out


def gradient_visibility(tau, w, h, dsf):
    """setup_target_visibility (sources/gradientIBR.cu:40-83)."""
    W, H = w * dsf, h * dsf
    vis = np.zeros(W * H, np.uint8)
    for v in views_of(np.zeros((tau.shape[0], 3, h, w), np.float32), tau, w, h, dsf):
        LIB.refg_setup_visibility_mask(W, H, _i(v.cells), 0, len(v.cells), v.ks, v.dsf, _f(v.tx), _f(v.ty), _u8(vis))
    return vis.reshape(H, W)


def u_gradient(views, tau, wg, w, h, dsf, sigma):
    """init_u_gradient (sources/gradientIBR.cu:833-920)."""
    W, H = w * dsf, h * dsf
    N, n = W * H, w * h
    wg = np.ascontiguousarray(wg, np.float32).reshape(-1, n)
    gx, gy, mask, norm = (np.zeros(N, np.float32) for _ in range(4))
    for k, v in enumerate(views_of(views, tau, w, h, dsf)):
        img = v.img.reshape(3, n)
        sx, sy = np.zeros(n, np.float32), np.zeros(n, np.float32)
        LIB.refg_compute_gradient(w, h, _f(img[0]), _f(img[1]), _f(img[2]), _f(sx), _f(sy))
        B = np.zeros_like(v.A)
        LIB.refg_set_B_bilinear(W, H, w, h, v.ks, _f(v.tx), _f(v.ty), _f(B))
        LIB.refg_deconvolution_rgb(W, H, _f(sx), _f(sy), _f(wg[k]), _i(v.cells), 0, len(v.cells), v.ks, v.dsf, _f(B),
                                   _f(v.tx), _f(v.ty), _f(gx), _f(gy), _f(mask), _f(norm))
    for a in (gx, gy, mask):
        LIB.ref_normalize(W, H, _f(a), _f(norm))
    LIB.ref_scale(W, H, _f(mask), np.float32(sigma) * np.float32(sigma))
    return gx.reshape(H, W), gy.reshape(H, W), mask.reshape(H, W)


def hole_fill(U, vis, max_iter=500):
    """hole_filling (sources/gradientIBR.cu:87-152) with its host float energy sum."""
    U = np.ascontiguousarray(U, np.float32)
    H, W = U.shape[1], U.shape[2]
    u = U.reshape(3, -1).copy()
    lap = np.zeros(H * W, np.float32)
    visf = np.ascontiguousarray(vis, np.uint8).ravel().copy()
    energy = np.float32(0.0)
    it = max_iter
    for k in range(max_iter):
        prev = energy
        for c in range(3):
            LIB.refg_compute_laplacian(W, H, _f(u[c]), _f(lap), _u8(visf))
            LIB.ref_add_to(W, H, _f(lap), _f(u[c]))
            LIB.ref_multiply_with(W, H, _f(lap), _f(u[c]))
            energy = np.float32(0.0)
            for e in lap:
                energy = np.float32(energy + e)
        if abs(prev - energy) < np.float32(1e-3):
            it = k + 1
            break
    return u.reshape(3, H, W), it


def poisson_jacobi(gx, gy, mask, U, iters=200):
    """poisson_jacobi (sources/gradientIBR.cu:923-1013) through the reference's compute_divergence, jacobi_z and
    jacobi_B kernels."""
    U = np.ascontiguousarray(U, np.float32).copy()
    H, W = U.shape[1], U.shape[2]
    gx, gy, mask = (np.ascontiguousarray(a, np.float32).copy() for a in (gx, gy, mask))
    LIB.refg_poisson_jacobi(W, H, iters, _f(gx), _f(gy), _f(mask), _f(U[0]), _f(U[1]), _f(U[2]))
    return U


if LIB is not None:
    LIB.ref_scale.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), F]
    LIB.ref_clamp.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), F, F]
    LIB.ref_add_scaled_to.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), F, C.POINTER(C.c_float)]
    LIB.ref_rof_dual_step.argtypes = [C.c_int, C.c_int, F] + [C.POINTER(C.c_float)] * 3
    LIB.ref_primal_prox.argtypes = [C.c_int, C.c_int, F, F] + [C.POINTER(C.c_float)] * 5
    LIB.ref_regularizer_weight.argtypes = [C.c_int, C.c_int, F, F, F] + [C.POINTER(C.c_float)] * 2
    LIB.ref_angular_weights.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), F,
                                        C.POINTER(C.c_float), C.POINTER(C.c_float), F, C.POINTER(C.c_float)]
    LIB.ref_overrelaxation.argtypes = [C.c_int, C.c_int, F, C.POINTER(C.c_float), C.POINTER(C.c_float)]
