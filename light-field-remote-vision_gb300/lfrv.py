"""Python binding of liblfrv.so (ctypes over the C ABI declared in include/lfrv.h).

The reference's entry points are C++ functions driven by a Config_data object:
    sr_synthesize_view(Config_data*)   -> Context.ibr_color(cfg, views, tau, dpart)
    IBR_gradient(Config_data*)         -> Context.ibr_gradient(cfg, views, tau, dpart)
    fromMVE2coco (GL warp export)      -> Context.warp(depth, cams, target)
Arrays are numpy float32, planar channel-major (V x C x h x w for view stacks, C x H x W for images).
Every call raises LfrvError with the library's message on a non-zero status. There is no CPU fallback:
loading fails if liblfrv.so is missing and every compute call needs a CUDA device.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("LFRV_LIB", _HERE / "liblfrv.so"))

OK, E_ARG, E_CUDA, E_NOMEM, E_IO, E_FORMAT, E_NONFINITE, E_TIMEOUT, E_NODEVICE = 0, -1, -2, -3, -4, -5, -6, -7, -8


class LfrvError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"lfrv status {status}: {message}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("dsf", C.c_int), ("nviews", C.c_int), ("nchannels", C.c_int),
                ("sigma_sensor", C.c_float), ("ugrad_threshold", C.c_float), ("lambda_", C.c_float),
                ("lambda_max_factor", C.c_float), ("dw_type", C.c_int), ("gw_type", C.c_int),
                ("dt_alpha", C.c_float), ("dt_beta", C.c_float), ("gradient_step", C.c_float),
                ("niter", C.c_int), ("nmeta_iter", C.c_int), ("faithful", C.c_int), ("early_exit", C.c_int),
                ("cg_max_iter", C.c_int), ("cg_gap_tol", C.c_double), ("hole_fill_iter", C.c_int),
                ("bf16_storage", C.c_int)]

    def copy(self) -> "Config":
        c = Config()
        C.pointer(c)[0] = self
        return c


class Camera(C.Structure):
    _fields_ = [("K", C.c_float * 9), ("R", C.c_float * 9), ("t", C.c_float * 3), ("width", C.c_int),
                ("height", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("outer_iterations", C.c_int), ("meta_iterations", C.c_int), ("hole_fill_iterations", C.c_int),
                ("stop_reason", C.c_int), ("energy", C.c_double), ("gap", C.c_double), ("seconds", C.c_double),
                ("kernel_launches", C.c_int), ("energy_trace", C.POINTER(C.c_double)), ("trace_capacity", C.c_int),
                ("trace_length", C.c_int)]

    @classmethod
    def with_trace(cls, capacity: int = 0) -> "Stats":
        """Statistics that also record the energy of every outer iteration (up to `capacity` entries)."""
        st = cls()
        if capacity > 0:
            st._trace_buf = np.zeros(capacity, np.float64)
            st.energy_trace = st._trace_buf.ctypes.data_as(C.POINTER(C.c_double))
            st.trace_capacity = capacity
        return st

    def trace(self) -> np.ndarray:
        """The recorded energy trace (empty when none was requested)."""
        buf = getattr(self, "_trace_buf", None)
        return np.zeros(0) if buf is None else buf[: self.trace_length].copy()

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "energy_trace"}


class SceneParams(C.Structure):
    _fields_ = [("grid", C.c_int), ("w", C.c_int), ("h", C.c_int), ("ss", C.c_int), ("dsf", C.c_int),
                ("baseline", C.c_double), ("nplanes", C.c_int), ("depths", C.c_double * 16), ("nbumps", C.c_int),
                ("bump_amp", C.c_double), ("bump_sigma_px", C.c_double), ("noise_sigma", C.c_double),
                ("focal_per_256", C.c_double), ("seed", C.c_uint64)]


class ViewJob(C.Structure):
    """lfrv_view_job: one target of a batch (device buffers, host cameras)."""
    _fields_ = [("cfg", C.POINTER(Config)), ("algorithm", C.c_int), ("d_views", C.c_void_p), ("d_depth", C.c_void_p),
                ("cams", C.POINTER(Camera)), ("target", C.POINTER(Camera)), ("d_out", C.c_void_p),
                ("stats", C.POINTER(Stats))]


_F = C.POINTER(C.c_float)
_U8 = C.POINTER(C.c_uint8)
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise LfrvError(E_NODEVICE, f"{LIB_PATH} not built; run __graft_entry__.build() first")
    lib = C.CDLL(str(LIB_PATH))
    lib.lfrv_last_error.restype = C.c_char_p
    lib.lfrv_version.restype = C.c_char_p
    lib.lfrv_psnr.restype = C.c_double
    lib.lfrv_psnr.argtypes = [C.c_int, C.c_int, _F, _F, C.c_int]
    return lib


LIB = _load()

# Every function declared in include/lfrv.h.
EXPORTED = [
    "lfrv_last_error", "lfrv_version", "lfrv_config_default", "lfrv_config_parse_file", "lfrv_config_set",
    "lfrv_config_get_string", "lfrv_config_get_int", "lfrv_ctx_create", "lfrv_ctx_destroy", "lfrv_ctx_set_stream",
    "lfrv_ctx_launch_count", "lfrv_ctx_profile", "lfrv_ctx_profile_read", "lfrv_depth_radial_to_ortho",
    "lfrv_depth_radial_to_ortho_dev", "lfrv_warp_from_depth", "lfrv_warp_from_depth_dev", "lfrv_warp", "lfrv_warp_dev", "lfrv_ibr_color", "lfrv_ibr_color_dev",
    "lfrv_ibr_gradient", "lfrv_ibr_gradient_dev", "lfrv_render_view", "lfrv_render_view_dev", "lfrv_render_views_dev",
    "lfrv_render_views", "lfrv_render_views_warm",
    "lfrv_video_camera", "lfrv_render_video_dev", "lfrv_mvei_read", "lfrv_depth_from_mve",
    "lfrv_warmstart_param_count", "lfrv_warmstart_create", "lfrv_warmstart_destroy", "lfrv_warmstart_get_params",
    "lfrv_warmstart_set_params", "lfrv_warmstart_features_dev", "lfrv_warmstart_forward_dev",
    "lfrv_warmstart_train_step_dev", "lfrv_warmstart_gradients_dev", "lfrv_render_view_warm_dev", "lfrv_render_views_warm_dev", "lfrv_conv_bf16_dev",
    "lfrv_set_conv_kernel",
    "lfrv_stage_weights",
    "lfrv_stage_visibility", "lfrv_stage_dataterm", "lfrv_stage_rof", "lfrv_stage_energy", "lfrv_stage_regularizer",
    "lfrv_stage_initial_image", "lfrv_stage_push_pull", "lfrv_stage_gradient_visibility", "lfrv_stage_hole_fill",
    "lfrv_stage_u_gradient", "lfrv_stage_cg", "lfrv_stage_poisson_jacobi", "lfrv_cg_solve_static", "lfrv_pfm_read", "lfrv_pfm_write", "lfrv_png_read", "lfrv_png_write",
    "lfrv_scene_params_preset",
    "lfrv_synth_scene", "lfrv_synth_scene_dev", "lfrv_psnr",
]


def _check(status: int) -> None:
    if status != OK:
        raise LfrvError(status, LIB.lfrv_last_error().decode(errors="replace"))


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous, "float32 C-contiguous array expected"
    return a.ctypes.data_as(_F)


def u8ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(_U8)


def f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


# ------------------------------------------------------------------ configuration
def default_config(**overrides) -> Config:
    cfg = Config()
    _check(LIB.lfrv_config_default(C.byref(cfg)))
    for k, v in overrides.items():
        setattr(cfg, "lambda_" if k == "lambda" else k, v)
    return cfg


def parse_config(path: str, cfg: Config | None = None) -> Config:
    cfg = cfg or default_config()
    _check(LIB.lfrv_config_parse_file(str(path).encode(), C.byref(cfg)))
    return cfg


def config_string(key: str) -> str:
    buf = C.create_string_buffer(1024)
    _check(LIB.lfrv_config_get_string(key.encode(), buf, C.c_size_t(len(buf))))
    return buf.value.decode()


# ------------------------------------------------------------------ synthetic scenes
@dataclass
class Scene:
    params: SceneParams
    views: np.ndarray   # V x 3 x h x w
    depth: np.ndarray   # V x 3 x h x w (z, dz/dx, dz/dy)
    cams: list          # V input cameras
    target: Camera
    gt: np.ndarray      # 3 x H x W


def scene_params(preset: int, **overrides) -> SceneParams:
    p = SceneParams()
    _check(LIB.lfrv_scene_params_preset(preset, C.byref(p)))
    for k, v in overrides.items():
        if k == "depths":
            for i, d in enumerate(v):
                p.depths[i] = d
            p.nplanes = len(v)
        else:
            setattr(p, k, v)
    return p


def synth_scene(p: SceneParams) -> Scene:
    V = p.grid * p.grid - 1
    h, w, H, W = p.h, p.w, p.h * p.dsf, p.w * p.dsf
    views = np.zeros((V, 3, h, w), np.float32)
    depth = np.zeros((V, 3, h, w), np.float32)
    cams = (Camera * (V + 1))()
    gt = np.zeros((3, H, W), np.float32)
    _check(LIB.lfrv_synth_scene(C.byref(p), fptr(views), fptr(depth), cams, fptr(gt)))
    return Scene(p, views, depth, [cams[i] for i in range(V)], cams[V], gt)


def cameras_array(cams) -> C.Array:
    arr = (Camera * len(cams))()
    for i, c in enumerate(cams):
        arr[i] = c
    return arr


def psnr(a: np.ndarray, b: np.ndarray, border: int = 2) -> float:
    a, b = f32(a), f32(b)
    return LIB.lfrv_psnr(a.shape[-1], a.shape[-2], fptr(a), fptr(b), border)


def pfm_read(path: str) -> np.ndarray:
    w, h, c = C.c_int(), C.c_int(), C.c_int()
    _check(LIB.lfrv_pfm_read(str(path).encode(), C.byref(w), C.byref(h), C.byref(c), None, C.c_size_t(0)))
    out = np.zeros((c.value, h.value, w.value), np.float32)
    _check(LIB.lfrv_pfm_read(str(path).encode(), C.byref(w), C.byref(h), C.byref(c), fptr(out),
                             C.c_size_t(out.size)))
    return out


def pfm_write(path: str, img: np.ndarray) -> None:
    img = f32(img)
    if img.ndim == 2:
        img = img[None]
    _check(LIB.lfrv_pfm_write(str(path).encode(), img.shape[2], img.shape[1], img.shape[0], fptr(img)))


CG_STATIC_MAX_PIXELS = 512 * 512


def cg_solve_static(stream: int, W: int, H: int, max_iter: int, gap_tol: float, d_gx: int, d_gy: int, d_U: int,
                    want_stats: bool = True):
    """Allocation-free corrected CG on device pointers (lfrv_cg_solve_static); returns (iterations, gap)."""
    it, gap = C.c_int(-1), C.c_double(float("nan"))
    _check(LIB.lfrv_cg_solve_static(C.c_void_p(stream or None), W, H, max_iter, C.c_double(gap_tol),
                                    C.c_void_p(d_gx), C.c_void_p(d_gy), C.c_void_p(d_U),
                                    C.byref(it) if want_stats else None, C.byref(gap) if want_stats else None))
    return it.value, gap.value


def mvei_read(path: str) -> np.ndarray:
    """MVE image (depth or normal map) as channels x h x w float32."""
    w, h, c = C.c_int(), C.c_int(), C.c_int()
    _check(LIB.lfrv_mvei_read(str(path).encode(), C.byref(w), C.byref(h), C.byref(c), None, C.c_size_t(0)))
    out = np.zeros((c.value, h.value, w.value), np.float32)
    _check(LIB.lfrv_mvei_read(str(path).encode(), C.byref(w), C.byref(h), C.byref(c), fptr(out),
                              C.c_size_t(out.size)))
    return out


def depth_from_mve(depth: np.ndarray, normal: np.ndarray, factor: int, invalid_depth: float = 1000.0) -> np.ndarray:
    """3 x (h0 factor) x (w0 factor) depth-map channels from an MVE depth plane (h0 x w0) and normal planes."""
    depth = f32(np.asarray(depth).reshape(-1, *np.asarray(depth).shape[-2:])[0])
    normal = f32(normal)
    h0, w0 = depth.shape
    out = np.zeros((3, h0 * factor, w0 * factor), np.float32)
    _check(LIB.lfrv_depth_from_mve(w0, h0, factor, fptr(depth), fptr(normal), C.c_float(invalid_depth), fptr(out)))
    return out


def video_camera(a: "Camera", b: "Camera", target: "Camera", frame: int) -> "Camera":
    """The IBR_video target camera of one frame (TargetView::move)."""
    out = Camera()
    _check(LIB.lfrv_video_camera(C.byref(a), C.byref(b), C.byref(target), frame, C.byref(out)))
    return out


def png_read(path: str) -> np.ndarray:
    """8-bit PNG as planar RGB floats in [0, 1] (value / 255, grey replicated), shape (3, h, w)."""
    w, h = C.c_int(), C.c_int()
    _check(LIB.lfrv_png_read(str(path).encode(), C.byref(w), C.byref(h), None, C.c_size_t(0)))
    out = np.zeros((3, h.value, w.value), np.float32)
    _check(LIB.lfrv_png_read(str(path).encode(), C.byref(w), C.byref(h), fptr(out), C.c_size_t(out.size)))
    return out


def png_write(path: str, img: np.ndarray) -> None:
    """Planar RGB floats (3, h, w) written as 8-bit RGB, clamp(int(v * 255), 0, 255) per channel."""
    img = f32(img)
    assert img.ndim == 3 and img.shape[0] == 3, "planar RGB (3, h, w) expected"
    _check(LIB.lfrv_png_write(str(path).encode(), img.shape[2], img.shape[1], fptr(img)))


# ------------------------------------------------------------------ contexts
class Context:
    """One device workspace (lfrv_ctx). Work is issued on `stream` (a cudaStream_t as int, 0 = default)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = C.c_void_p()
        _check(LIB.lfrv_ctx_create(C.byref(self._h), device))
        if stream:
            self.set_stream(stream)

    def close(self) -> None:
        if self._h:
            LIB.lfrv_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream: int) -> None:
        _check(LIB.lfrv_ctx_set_stream(self._h, C.c_void_p(stream)))

    def launch_count(self, reset: bool = False) -> int:
        n = C.c_longlong()
        _check(LIB.lfrv_ctx_launch_count(self._h, C.byref(n), int(reset)))
        return n.value

    def profile_enable(self, on: bool = True) -> None:
        _check(LIB.lfrv_ctx_profile(self._h, int(on)))

    def profile(self) -> dict:
        """{kernel launcher name: (total device ms, launches)} since profile_enable(True)."""
        out = {}
        name = C.create_string_buffer(128)
        ms, cnt = C.c_double(), C.c_longlong()
        i = 0
        while True:
            st = LIB.lfrv_ctx_profile_read(self._h, i, name, C.c_size_t(len(name)), C.byref(ms), C.byref(cnt))
            if st != OK:
                break
            out[name.value.decode()] = (ms.value, cnt.value)
            i += 1
        return out

    # ---- warp stage
    def warp_from_depth(self, depth: np.ndarray, cams, target: Camera, dsf: int, faithful: bool = True):
        """Warps (V x 3 x h x w) from depth maps (V x C x h x w, plane 0 = z) without the GL pipeline."""
        depth = f32(depth)
        V, ch, h, w = depth.shape
        tau = np.zeros((V, 3, h, w), np.float32)
        _check(LIB.lfrv_warp_from_depth(self._h, V, w, h, dsf, fptr(depth), ch, cameras_array(cams), C.byref(target),
                                        int(faithful), fptr(tau)))
        return tau

    def depth_radial_to_ortho(self, depth: np.ndarray, cams) -> np.ndarray:
        """Radial to orthographic depth maps (V x 3 x h x w); returns a converted copy."""
        d = f32(depth).copy()
        V, _, h, w = d.shape
        _check(LIB.lfrv_depth_radial_to_ortho(self._h, V, w, h, cameras_array(cams), fptr(d)))
        return d

    def warp(self, depth: np.ndarray, cams, target: Camera):
        depth = f32(depth)
        V, _, h, w = depth.shape
        tau = np.zeros((V, 3, h, w), np.float32)
        dpart = np.zeros((V, 3, h, w), np.float32)
        zbuf = np.zeros((target.height, target.width), np.float32)
        _check(LIB.lfrv_warp(self._h, V, w, h, fptr(depth), cameras_array(cams), C.byref(target), fptr(tau),
                             fptr(dpart), fptr(zbuf)))
        return tau, dpart, zbuf

    def warp_dev(self, nviews: int, w: int, h: int, d_depth: int, cams, target: Camera, d_tau: int, d_dpart: int,
                 d_zbuf: int = 0) -> None:
        _check(LIB.lfrv_warp_dev(self._h, nviews, w, h, C.c_void_p(d_depth), cameras_array(cams), C.byref(target),
                                 C.c_void_p(d_tau), C.c_void_p(d_dpart), C.c_void_p(d_zbuf or None)))

    # ---- solvers
    def _solve(self, fn, cfg: Config, views, tau, dpart, init=None, trace: int = 0):
        views, tau = f32(views), f32(tau)
        dpart = None if dpart is None else f32(dpart)
        init = None if init is None else f32(init)
        H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
        out = np.zeros((3, H, W), np.float32)
        st = Stats.with_trace(trace)
        _check(fn(self._h, C.byref(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(dpart), fptr(init), fptr(out),
                  C.byref(st)))
        return out, st

    def ibr_color(self, cfg: Config, views, tau, dpart, init=None, trace: int = 0):
        return self._solve(LIB.lfrv_ibr_color, cfg, views, tau, dpart, init, trace)

    def ibr_gradient(self, cfg: Config, views, tau, dpart, init=None, trace: int = 0):
        return self._solve(LIB.lfrv_ibr_gradient, cfg, views, tau, dpart, init, trace)

    def solve_dev(self, algorithm: int, cfg: Config, d_views: int, d_tau: int, tau_channels: int, d_dpart: int,
                  d_out: int, d_init: int = 0, trace: int = 0) -> Stats:
        st = Stats.with_trace(trace)
        fn = LIB.lfrv_ibr_color_dev if algorithm == 0 else LIB.lfrv_ibr_gradient_dev
        _check(fn(self._h, C.byref(cfg), C.c_void_p(d_views), C.c_void_p(d_tau), tau_channels,
                  C.c_void_p(d_dpart or None), C.c_void_p(d_init or None), C.c_void_p(d_out), C.byref(st)))
        return st

    def render_view_dev(self, cfg: Config, algorithm: int, d_views: int, d_depth: int, cams, target: Camera,
                        d_out: int, trace: int = 0) -> Stats:
        st = Stats.with_trace(trace)
        _check(LIB.lfrv_render_view_dev(self._h, C.byref(cfg), algorithm, C.c_void_p(d_views), C.c_void_p(d_depth),
                                        cameras_array(cams), C.byref(target), C.c_void_p(d_out), C.byref(st)))
        return st

    def synth_scene_dev(self, p: SceneParams, d_views: int = 0, d_depth: int = 0, d_gt: int = 0):
        """The scene of `p` generated on the GPU into device buffers (views and depth V x 3 x h x w, gt 3 x H x W;
        0 skips one); returns (input cameras, target camera)."""
        V = p.grid * p.grid - 1
        cams = (Camera * (V + 1))()
        _check(LIB.lfrv_synth_scene_dev(self._h, C.byref(p), C.c_void_p(d_views or None), C.c_void_p(d_depth or None),
                                        cams, C.c_void_p(d_gt or None)))
        return [cams[i] for i in range(V)], cams[V]

    def render_video_dev(self, cfg: Config, algorithm: int, d_views: int, d_depth: int, cams, cam_a: int, cam_b: int,
                         target: Camera, first_frame: int, nframes: int, d_out: int) -> list:
        """IBR_video frames first_frame .. first_frame + nframes - 1 as one batch; d_out: nframes x 3 x H x W."""
        stats = (Stats * nframes)()
        _check(LIB.lfrv_render_video_dev(self._h, C.byref(cfg), algorithm, C.c_void_p(d_views), C.c_void_p(d_depth),
                                         cameras_array(cams), cam_a, cam_b, C.byref(target), first_frame, nframes,
                                         C.c_void_p(d_out), stats))
        return list(stats)

    def render_views(self, jobs, net: "WarmStart | None" = None, trace: int = 0) -> list:
        """Batched targets from host buffers (lfrv_render_views / lfrv_render_views_warm): each job's d_views,
        d_depth and d_out are HOST pointers (ints); shared inputs are uploaded once. Returns one Stats per job."""
        return self.render_views_dev(jobs, net, trace, host=True)

    def render_views_dev(self, jobs, net: "WarmStart | None" = None, trace: int = 0, host: bool = False) -> list:
        """Batched targets: jobs is a list of dicts with cfg, algorithm, d_views, d_depth, cams, target, d_out
        (device pointers as ints). With a warm-start network the IBR_gradient jobs are seeded by it
        (lfrv_render_views_warm_dev). Returns one Stats per job (with `trace` entries of energy trace each)."""
        arr = (ViewJob * len(jobs))()
        keep = []
        stats = [Stats.with_trace(trace) for _ in jobs]
        for i, j in enumerate(jobs):
            cams = cameras_array(j["cams"])
            tgt = Camera()
            C.pointer(tgt)[0] = j["target"]
            keep += [cams, tgt, j["cfg"]]
            arr[i] = ViewJob(C.pointer(j["cfg"]), int(j["algorithm"]), C.c_void_p(j["d_views"]), C.c_void_p(j["d_depth"]),
                             C.cast(cams, C.POINTER(Camera)), C.pointer(tgt), C.c_void_p(j["d_out"]),
                             C.pointer(stats[i]))
        if net is None:
            _check((LIB.lfrv_render_views if host else LIB.lfrv_render_views_dev)(self._h, arr, len(jobs)))
        else:
            fn = LIB.lfrv_render_views_warm if host else LIB.lfrv_render_views_warm_dev
            _check(fn(self._h, net._h, arr, len(jobs)))
        return stats

    def render_view(self, cfg: Config, algorithm: int, views, depth, cams, target: Camera, out=None,
                    trace: int = 0):
        """Host-buffer pipeline (copies inside the call). views/depth/out may be numpy arrays or host pointers."""
        st = Stats.with_trace(trace)
        views_p = views if isinstance(views, int) else f32(views).ctypes.data
        depth_p = depth if isinstance(depth, int) else f32(depth).ctypes.data
        if out is None:
            out = np.zeros((3, cfg.h * cfg.dsf, cfg.w * cfg.dsf), np.float32)
        out_p = out if isinstance(out, int) else out.ctypes.data
        _check(LIB.lfrv_render_view(self._h, C.byref(cfg), algorithm, C.c_void_p(views_p), C.c_void_p(depth_p),
                                    cameras_array(cams), C.byref(target), C.c_void_p(out_p), C.byref(st)))
        return out, st

    def warmstart_features_dev(self, cfg: Config, d_views: int, d_depth: int, cams, target: Camera, d_input: int,
                               d_u0: int, d_solution: int = 0) -> Stats:
        st = Stats()
        _check(LIB.lfrv_warmstart_features_dev(self._h, C.byref(cfg), C.c_void_p(d_views), C.c_void_p(d_depth),
                                               cameras_array(cams), C.byref(target), C.c_void_p(d_input),
                                               C.c_void_p(d_u0 or None), C.c_void_p(d_solution or None),
                                               C.byref(st)))
        return st

    def conv_bf16_dev(self, mode: int, batch: int, H: int, W: int, Cin: int, Cout: int, ks: int, stride: int,
                      d_x: int, d_dy: int, d_w: int, d_out: int) -> None:
        _check(LIB.lfrv_conv_bf16_dev(self._h, mode, batch, H, W, Cin, Cout, ks, stride, C.c_void_p(d_x or None),
                                      C.c_void_p(d_dy or None), C.c_void_p(d_w), C.c_void_p(d_out)))

    # ---- stage calls (parity tests)
    def stage_visibility(self, cfg: Config, tau):
        tau = f32(tau)
        H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
        cov = np.zeros((H, W), np.float32)
        vis = np.zeros((H, W), np.uint8)
        _check(LIB.lfrv_stage_visibility(self._h, C.byref(cfg), fptr(tau), tau.shape[1], fptr(cov), u8ptr(vis)))
        return cov, vis

    def stage_weights(self, cfg: Config, views, tau, dpart, U, vis, gx, gy):
        views, tau, dpart, U = f32(views), f32(tau), f32(dpart), f32(U)
        vis = np.ascontiguousarray(vis, np.uint8)
        gx, gy = f32(gx).copy(), f32(gy).copy()
        wgt = np.zeros((cfg.nviews, cfg.h, cfg.w), np.float32)
        _check(LIB.lfrv_stage_weights(self._h, C.byref(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(dpart),
                                      fptr(U), u8ptr(vis), fptr(gx), fptr(gy), fptr(wgt)))
        return gx, gy, wgt

    def stage_dataterm(self, cfg: Config, views, tau, weights, U):
        views, tau, weights, U = f32(views), f32(tau), f32(weights), f32(U)
        G = np.zeros_like(U)
        F = np.zeros_like(U)
        _check(LIB.lfrv_stage_dataterm(self._h, C.byref(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights),
                                       fptr(U), fptr(G), fptr(F)))
        return G, F

    def stage_rof(self, niter: int, tau: float, sigma: float, lam: float, F, g, U, P):
        F, g = f32(F), f32(g)
        U, P = f32(U).copy(), f32(P).copy()
        H, W = U.shape[1], U.shape[2]
        _check(LIB.lfrv_stage_rof(self._h, W, H, niter, C.c_float(tau), C.c_float(sigma), C.c_float(lam), fptr(F),
                                  fptr(g), fptr(U), fptr(P)))
        return U, P

    def stage_energy(self, cfg: Config, views, tau, weights, U, vis):
        views, tau, weights, U = f32(views), f32(tau), f32(weights), f32(U)
        vis = np.ascontiguousarray(vis, np.uint8)
        e, et, ed = C.c_double(), C.c_double(), C.c_double()
        _check(LIB.lfrv_stage_energy(self._h, C.byref(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights),
                                     fptr(U), u8ptr(vis), C.byref(e), C.byref(et), C.byref(ed)))
        return e.value, et.value, ed.value

    def stage_regularizer(self, cfg: Config, tau, weights, norm_in=None):
        tau, weights = f32(tau), f32(weights)
        H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
        norm_out = np.zeros((H, W), np.float32)
        g = np.zeros((H, W), np.float32)
        _check(LIB.lfrv_stage_regularizer(self._h, C.byref(cfg), fptr(tau), tau.shape[1], fptr(weights),
                                          fptr(None if norm_in is None else f32(norm_in)), fptr(norm_out), fptr(g)))
        return norm_out, g

    def stage_initial_image(self, cfg: Config, views, tau, weights):
        views, tau, weights = f32(views), f32(tau), f32(weights)
        H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
        U = np.zeros((3, H, W), np.float32)
        norm = np.zeros((H, W), np.float32)
        _check(LIB.lfrv_stage_initial_image(self._h, C.byref(cfg), fptr(views), fptr(tau), tau.shape[1],
                                            fptr(weights), fptr(U), fptr(norm)))
        return U, norm

    def stage_push_pull(self, U, vis, faithful: bool = True):
        U = f32(U).copy()
        vis = np.ascontiguousarray(vis, np.uint8)
        _check(LIB.lfrv_stage_push_pull(self._h, U.shape[2], U.shape[1], int(faithful), u8ptr(vis), fptr(U)))
        return U

    def stage_gradient_visibility(self, cfg: Config, tau):
        tau = f32(tau)
        vis = np.zeros((cfg.h * cfg.dsf, cfg.w * cfg.dsf), np.uint8)
        _check(LIB.lfrv_stage_gradient_visibility(self._h, C.byref(cfg), fptr(tau), tau.shape[1], u8ptr(vis)))
        return vis

    def stage_hole_fill(self, U, vis, max_iter: int = 500):
        U = f32(U).copy()
        vis = np.ascontiguousarray(vis, np.uint8)
        it = C.c_int()
        _check(LIB.lfrv_stage_hole_fill(self._h, U.shape[2], U.shape[1], max_iter, u8ptr(vis), fptr(U),
                                        C.byref(it)))
        return U, it.value

    def stage_u_gradient(self, cfg: Config, views, tau, weights):
        views, tau, weights = f32(views), f32(tau), f32(weights)
        H, W = cfg.h * cfg.dsf, cfg.w * cfg.dsf
        gx, gy, mask = (np.zeros((H, W), np.float32) for _ in range(3))
        _check(LIB.lfrv_stage_u_gradient(self._h, C.byref(cfg), fptr(views), fptr(tau), tau.shape[1], fptr(weights),
                                         fptr(gx), fptr(gy), fptr(mask)))
        return gx, gy, mask

    def stage_poisson_jacobi(self, gx, gy, mask, U, iterations: int = 200):
        """poisson_jacobi: `iterations` Jacobi sweeps on a copy of U (3 x H x W)."""
        gx, gy, mask = f32(gx), f32(gy), f32(mask)
        U = f32(U).copy()
        _check(LIB.lfrv_stage_poisson_jacobi(self._h, U.shape[2], U.shape[1], iterations, fptr(gx), fptr(gy),
                                             fptr(mask), fptr(U)))
        return U

    def stage_cg(self, gx, gy, U, faithful: bool, max_iter: int = 500, gap_tol: float = 1e-4):
        gx, gy = f32(gx), f32(gy)
        U = f32(U).copy()
        it, gap = C.c_int(), C.c_double()
        _check(LIB.lfrv_stage_cg(self._h, U.shape[2], U.shape[1], int(faithful), max_iter, C.c_double(gap_tol),
                                 fptr(gx), fptr(gy), fptr(U), C.byref(it), C.byref(gap)))
        return U, it.value, gap.value


# ------------------------------------------------------------------ learned warm start
WARMSTART_CHANNELS = 48


def set_conv_kernel(which: int) -> None:
    """0 (default): TMA, resident-tile or gather kernel as they apply; 1: no TMA kernel; 2: gather only."""
    _check(LIB.lfrv_set_conv_kernel(which))


def warmstart_param_count() -> int:
    return int(LIB.lfrv_warmstart_param_count())


class WarmStart:
    """The learned warm start of IBR_gradient (lfrv_warmstart_*). Tensors are device pointers (ints): inputs
    batch x H x W x 48 BF16, u0 / targets / predictions batch x 3 x H x W float32."""

    def __init__(self, ctx: "Context", seed: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        _check(LIB.lfrv_warmstart_create(ctx._h, C.c_ulonglong(seed), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            LIB.lfrv_warmstart_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(warmstart_param_count(), np.float32)
        _check(LIB.lfrv_warmstart_get_params(self._h, fptr(out)))
        return out

    def set_params(self, params: np.ndarray) -> None:
        params = f32(params)
        assert params.size == warmstart_param_count()
        _check(LIB.lfrv_warmstart_set_params(self._h, fptr(params)))

    def forward_dev(self, batch: int, H: int, W: int, d_input: int, d_u0: int, d_pred: int) -> None:
        _check(LIB.lfrv_warmstart_forward_dev(self._h, batch, H, W, C.c_void_p(d_input), C.c_void_p(d_u0),
                                              C.c_void_p(d_pred)))

    def train_step_dev(self, batch: int, H: int, W: int, d_input: int, d_u0: int, d_target: int,
                       lr: float) -> float:
        loss = C.c_double()
        _check(LIB.lfrv_warmstart_train_step_dev(self._h, batch, H, W, C.c_void_p(d_input), C.c_void_p(d_u0),
                                                 C.c_void_p(d_target), C.c_float(lr), C.byref(loss)))
        return loss.value

    def gradients_dev(self, batch: int, H: int, W: int, d_input: int, d_u0: int, d_target: int):
        loss = C.c_double()
        g = np.zeros(warmstart_param_count(), np.float32)
        _check(LIB.lfrv_warmstart_gradients_dev(self._h, batch, H, W, C.c_void_p(d_input), C.c_void_p(d_u0),
                                                C.c_void_p(d_target), C.byref(loss), fptr(g)))
        return loss.value, g

    def render_view_dev(self, cfg: Config, d_views: int, d_depth: int, cams, target: Camera, d_out: int) -> Stats:
        st = Stats()
        _check(LIB.lfrv_render_view_warm_dev(self.ctx._h, self._h, C.byref(cfg), C.c_void_p(d_views),
                                             C.c_void_p(d_depth), cameras_array(cams), C.byref(target),
                                             C.c_void_p(d_out), C.byref(st)))
        return st


def _declare() -> None:
    vp = C.c_void_p
    LIB.lfrv_ctx_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    LIB.lfrv_ctx_destroy.argtypes = [vp]
    LIB.lfrv_ctx_set_stream.argtypes = [vp, vp]
    LIB.lfrv_ctx_launch_count.argtypes = [vp, C.POINTER(C.c_longlong), C.c_int]
    LIB.lfrv_ctx_profile.argtypes = [vp, C.c_int]
    LIB.lfrv_ctx_profile_read.argtypes = [vp, C.c_int, C.c_char_p, C.c_size_t, _D, C.POINTER(C.c_longlong)]
    LIB.lfrv_warp.argtypes = [vp, C.c_int, C.c_int, C.c_int, _F, C.POINTER(Camera), C.POINTER(Camera), _F, _F, _F]
    LIB.lfrv_warp_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, C.POINTER(Camera), C.POINTER(Camera), vp, vp, vp]
    for name in ("lfrv_ibr_color", "lfrv_ibr_gradient"):
        getattr(LIB, name).argtypes = [vp, C.POINTER(Config), _F, _F, C.c_int, _F, _F, _F, C.POINTER(Stats)]
    for name in ("lfrv_ibr_color_dev", "lfrv_ibr_gradient_dev"):
        getattr(LIB, name).argtypes = [vp, C.POINTER(Config), vp, vp, C.c_int, vp, vp, vp, C.POINTER(Stats)]
    LIB.lfrv_render_view_dev.argtypes = [vp, C.POINTER(Config), C.c_int, vp, vp, C.POINTER(Camera),
                                         C.POINTER(Camera), vp, C.POINTER(Stats)]
    LIB.lfrv_render_view.argtypes = [vp, C.POINTER(Config), C.c_int, vp, vp, C.POINTER(Camera), C.POINTER(Camera),
                                     vp, C.POINTER(Stats)]
    LIB.lfrv_stage_rof.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _F, _F, _F, _F]
    LIB.lfrv_stage_cg.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _F, _F, _F, _I, _D]
    LIB.lfrv_stage_poisson_jacobi.argtypes = [vp, C.c_int, C.c_int, C.c_int, _F, _F, _F, _F]
    LIB.lfrv_stage_push_pull.argtypes = [vp, C.c_int, C.c_int, C.c_int, _U8, _F]
    LIB.lfrv_stage_hole_fill.argtypes = [vp, C.c_int, C.c_int, C.c_int, _U8, _F, _I]
    LIB.lfrv_synth_scene.argtypes = [C.POINTER(SceneParams), _F, _F, C.POINTER(Camera), _F]
    LIB.lfrv_synth_scene_dev.argtypes = [vp, C.POINTER(SceneParams), vp, vp, C.POINTER(Camera), vp]
    LIB.lfrv_scene_params_preset.argtypes = [C.c_int, C.POINTER(SceneParams)]
    LIB.lfrv_config_get_string.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
    LIB.lfrv_pfm_read.argtypes = [C.c_char_p, _I, _I, _I, _F, C.c_size_t]
    LIB.lfrv_pfm_write.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, _F]
    LIB.lfrv_warp_from_depth.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, _F, C.c_int, C.POINTER(Camera),
                                         C.POINTER(Camera), C.c_int, _F]
    LIB.lfrv_warp_from_depth_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int, C.POINTER(Camera),
                                             C.POINTER(Camera), C.c_int, vp]
    LIB.lfrv_depth_radial_to_ortho.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(Camera), _F]
    LIB.lfrv_depth_radial_to_ortho_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(Camera), vp]
    LIB.lfrv_render_views_dev.argtypes = [vp, C.POINTER(ViewJob), C.c_int]
    LIB.lfrv_render_views.argtypes = [vp, C.POINTER(ViewJob), C.c_int]
    LIB.lfrv_video_camera.argtypes = [C.POINTER(Camera)] * 3 + [C.c_int, C.POINTER(Camera)]
    LIB.lfrv_render_video_dev.argtypes = [vp, C.POINTER(Config), C.c_int, vp, vp, C.POINTER(Camera), C.c_int,
                                          C.c_int, C.POINTER(Camera), C.c_int, C.c_int, vp, C.POINTER(Stats)]
    LIB.lfrv_mvei_read.argtypes = [C.c_char_p, _I, _I, _I, _F, C.c_size_t]
    LIB.lfrv_depth_from_mve.argtypes = [C.c_int, C.c_int, C.c_int, _F, _F, C.c_float, _F]
    LIB.lfrv_render_views_warm.argtypes = [vp, vp, C.POINTER(ViewJob), C.c_int]
    LIB.lfrv_cg_solve_static.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, vp, vp, vp, _I, _D]
    LIB.lfrv_png_read.argtypes = [C.c_char_p, _I, _I, _F, C.c_size_t]
    LIB.lfrv_png_write.argtypes = [C.c_char_p, C.c_int, C.c_int, _F]
    LIB.lfrv_warmstart_param_count.restype = C.c_longlong
    LIB.lfrv_warmstart_param_count.argtypes = []
    LIB.lfrv_warmstart_create.argtypes = [vp, C.c_ulonglong, C.POINTER(C.c_void_p)]
    LIB.lfrv_warmstart_destroy.argtypes = [vp]
    LIB.lfrv_warmstart_destroy.restype = None
    LIB.lfrv_warmstart_get_params.argtypes = [vp, _F]
    LIB.lfrv_warmstart_set_params.argtypes = [vp, _F]
    LIB.lfrv_warmstart_features_dev.argtypes = [vp, C.POINTER(Config), vp, vp, C.POINTER(Camera), C.POINTER(Camera),
                                                vp, vp, vp, C.POINTER(Stats)]
    LIB.lfrv_warmstart_forward_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
    LIB.lfrv_warmstart_train_step_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_float, _D]
    LIB.lfrv_warmstart_gradients_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, _D, _F]
    LIB.lfrv_render_view_warm_dev.argtypes = [vp, vp, C.POINTER(Config), vp, vp, C.POINTER(Camera),
                                              C.POINTER(Camera), vp, C.POINTER(Stats)]
    LIB.lfrv_render_views_warm_dev.argtypes = [vp, vp, C.POINTER(ViewJob), C.c_int]
    LIB.lfrv_set_conv_kernel.argtypes = [C.c_int]
    LIB.lfrv_conv_bf16_dev.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       vp, vp, vp, vp]


_declare()
