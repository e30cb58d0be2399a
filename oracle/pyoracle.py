"""ctypes binding of oracle/liblfrv_oracle.so -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg use this module, as the checker
(or the timed CPU baseline). prec=0 selects the FP64 oracle, prec=1 the FP32 mirror of the reference's
float arithmetic.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(_HERE.parent / "light-field-remote-vision_gb300"))
import lfrv  # noqa: E402  (struct layouts shared with the product's header)

LIB = C.CDLL(str(Path(os.environ.get("LFRV_ORACLE_LIB", _HERE / "liblfrv_oracle.so"))))
_F = C.POINTER(C.c_float)
_U8 = C.POINTER(C.c_uint8)
f32, fptr, u8ptr = lfrv.f32, lfrv.fptr, lfrv.u8ptr
LIB.orc_cg_energy.restype = C.c_double


def _cfg(cfg):
    return C.byref(cfg)


def ibr_color(cfg, views, tau, dpart, init=None, prec=0, trace=0):
    views, tau = f32(views), f32(tau)
    out = np.zeros((3, cfg.h * cfg.dsf, cfg.w * cfg.dsf), np.float32)
    st = lfrv.Stats.with_trace(trace)
    LIB.orc_ibr_color(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(None if dpart is None else f32(dpart)),
                      fptr(None if init is None else f32(init)), fptr(out), C.byref(st))
    return out, st


def ibr_gradient(cfg, views, tau, dpart, init=None, prec=0, trace=0):
    views, tau = f32(views), f32(tau)
    out = np.zeros((3, cfg.h * cfg.dsf, cfg.w * cfg.dsf), np.float32)
    st = lfrv.Stats.with_trace(trace)
    LIB.orc_ibr_gradient(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1],
                         fptr(None if dpart is None else f32(dpart)), fptr(None if init is None else f32(init)),
                         fptr(out), C.byref(st))
    return out, st


def stage_visibility(cfg, tau, prec=0):
    tau = f32(tau)
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    cov = np.zeros((H, W), np.float32)
    vis = np.zeros((H, W), np.uint8)
    LIB.orc_stage_visibility(prec, _cfg(cfg), fptr(tau), tau.shape[1], fptr(cov), u8ptr(vis))
    return cov, vis


def stage_weights(cfg, views, tau, dpart, U, vis, gx, gy, prec=0):
    views, tau, dpart, U = f32(views), f32(tau), f32(dpart), f32(U)
    vis = np.ascontiguousarray(vis, np.uint8)
    gx, gy = f32(gx).copy(), f32(gy).copy()
    wgt = np.zeros((cfg.nviews, cfg.h, cfg.w), np.float32)
    LIB.orc_stage_weights(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(dpart), fptr(U), u8ptr(vis),
                          fptr(gx), fptr(gy), fptr(wgt))
    return gx, gy, wgt


def stage_dataterm(cfg, views, tau, weights, U, prec=0):
    views, tau, weights, U = f32(views), f32(tau), f32(weights), f32(U)
    G = np.zeros_like(U)
    F = np.zeros_like(U)
    LIB.orc_stage_dataterm(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights), fptr(U), fptr(G),
                           fptr(F))
    return G, F


def stage_rof(niter, tau, sigma, lam, F, g, U, P, prec=0):
    F, g = f32(F), f32(g)
    U, P = f32(U).copy(), f32(P).copy()
    LIB.orc_stage_rof(prec, U.shape[2], U.shape[1], niter, C.c_float(tau), C.c_float(sigma), C.c_float(lam), fptr(F),
                      fptr(g), fptr(U), fptr(P))
    return U, P


def stage_energy(cfg, views, tau, weights, U, vis, prec=0):
    views, tau, weights, U = f32(views), f32(tau), f32(weights), f32(U)
    vis = np.ascontiguousarray(vis, np.uint8)
    e, et, ed = C.c_double(), C.c_double(), C.c_double()
    LIB.orc_stage_energy(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights), fptr(U), u8ptr(vis),
                         C.byref(e), C.byref(et), C.byref(ed))
    return e.value, et.value, ed.value


def stage_regularizer(cfg, tau, weights, norm_in=None, prec=0):
    tau, weights = f32(tau), f32(weights)
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    norm_out = np.zeros((H, W), np.float32)
    g = np.zeros((H, W), np.float32)
    LIB.orc_stage_regularizer(prec, _cfg(cfg), fptr(tau), tau.shape[1], fptr(weights),
                              fptr(None if norm_in is None else f32(norm_in)), fptr(norm_out), fptr(g))
    return norm_out, g


def stage_initial_image(cfg, views, tau, weights, prec=0):
    views, tau, weights = f32(views), f32(tau), f32(weights)
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    U = np.zeros((3, H, W), np.float32)
    norm = np.zeros((H, W), np.float32)
    LIB.orc_stage_initial_image(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights), fptr(U),
                                fptr(norm))
    return U, norm


def stage_push_pull(U, vis, faithful=True, prec=0):
    U = f32(U).copy()
    vis = np.ascontiguousarray(vis, np.uint8)
    LIB.orc_stage_push_pull(prec, U.shape[2], U.shape[1], int(faithful), u8ptr(vis), fptr(U))
    return U


def stage_gradient_visibility(cfg, tau, prec=0):
    tau = f32(tau)
    vis = np.zeros((cfg.h * cfg.dsf, cfg.w * cfg.dsf), np.uint8)
    LIB.orc_stage_gradient_visibility(prec, _cfg(cfg), fptr(tau), tau.shape[1], u8ptr(vis))
    return vis


def stage_hole_fill(U, vis, max_iter=500, prec=0):
    U = f32(U).copy()
    vis = np.ascontiguousarray(vis, np.uint8)
    it = C.c_int()
    LIB.orc_stage_hole_fill(prec, U.shape[2], U.shape[1], max_iter, u8ptr(vis), fptr(U), C.byref(it))
    return U, it.value


def stage_u_gradient(cfg, views, tau, weights, prec=0):
    views, tau, weights = f32(views), f32(tau), f32(weights)
    H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
    gx, gy, mask = (np.zeros((H, W), np.float32) for _ in range(3))
    LIB.orc_stage_u_gradient(prec, _cfg(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights), fptr(gx),
                             fptr(gy), fptr(mask))
    return gx, gy, mask


def stage_cg(gx, gy, U, faithful, max_iter=500, gap_tol=1e-4, prec=0):
    gx, gy = f32(gx), f32(gy)
    U = f32(U).copy()
    it, gap = C.c_int(), C.c_double()
    LIB.orc_stage_cg(prec, U.shape[2], U.shape[1], int(faithful), max_iter, C.c_double(gap_tol), fptr(gx), fptr(gy),
                     fptr(U), C.byref(it), C.byref(gap))
    return U, it.value, gap.value


def stage_poisson_jacobi(gx, gy, mask, U, iters=200, prec=0):
    """poisson_jacobi (sources/gradientIBR.cu:923-1013): `iters` Jacobi sweeps on U (3 x H x W) for the gradient
    constraint (gx, gy) and the target mask."""
    gx, gy, mask = f32(gx), f32(gy), f32(mask)
    U = f32(U).copy()
    LIB.orc_stage_poisson_jacobi(prec, U.shape[2], U.shape[1], iters, fptr(gx), fptr(gy), fptr(mask), fptr(U))
    return U


def cg_energy(U, U0, gx, gy):
    U, U0, gx, gy = f32(U), f32(U0), f32(gx), f32(gy)
    return LIB.orc_cg_energy(U.shape[2], U.shape[1], fptr(U), fptr(U0), fptr(gx), fptr(gy))


def warp(depth, cams, target):
    depth = f32(depth)
    V, _, h, w = depth.shape
    tau = np.zeros((V, 3, h, w), np.float32)
    dpart = np.zeros((V, 3, h, w), np.float32)
    zbuf = np.zeros((target.height, target.width), np.float32)
    LIB.orc_warp(V, w, h, fptr(depth), lfrv.cameras_array(cams), C.byref(target), fptr(tau), fptr(dpart), fptr(zbuf))
    return tau, dpart, zbuf


def warp_from_depth(depth, cams, target, dsf, faithful=1):
    """import_warps_from_depth: V x 3 x h x w warps from V x C x h x w depth maps (plane 0 = z)."""
    depth = f32(depth)
    V, ch, h, w = depth.shape
    tau = np.zeros((V, 3, h, w), np.float32)
    LIB.orc_warp_from_depth(V, w, h, dsf, fptr(depth), ch, lfrv.cameras_array(cams), C.byref(target), int(faithful),
                            fptr(tau))
    return tau


def depth_radial_to_ortho(depth, cams):
    """fromRadial2Ortho.frag on V x 3 x h x w depth maps (returns a converted copy)."""
    d = f32(depth).copy()
    V, _, h, w = d.shape
    LIB.orc_depth_radial_to_ortho(V, w, h, lfrv.cameras_array(cams), fptr(d))
    return d


def footprint(tx, ty, dsf, W, H, prec=1):
    x0, y0 = C.c_int(), C.c_int()
    A = np.zeros(25, np.float32)
    LIB.orc_footprint(prec, C.c_float(tx), C.c_float(ty), dsf, W, H, C.byref(x0), C.byref(y0), fptr(A))
    ks = dsf + 1
    return x0.value, y0.value, A[: ks * ks].reshape(ks, ks)


def gaussian_blur(img, prec=0):
    img = f32(img)
    out = np.zeros_like(img)
    LIB.orc_gaussian_blur(prec, img.shape[1], img.shape[0], fptr(img), fptr(out))
    return out


def sobel(rgb, vis=None, gx=None, gy=None, prec=0):
    rgb = f32(rgb)
    H, W = rgb.shape[1], rgb.shape[2]
    gx = np.zeros((H, W), np.float32) if gx is None else f32(gx).copy()
    gy = np.zeros((H, W), np.float32) if gy is None else f32(gy).copy()
    LIB.orc_sobel(prec, W, H, fptr(rgb), u8ptr(None if vis is None else np.ascontiguousarray(vis, np.uint8)),
                  fptr(gx), fptr(gy))
    return gx, gy
