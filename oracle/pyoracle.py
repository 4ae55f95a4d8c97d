"""Python driver of the CPU oracle (oracle/_build/liboracle.so) and of the compiled reference
shaders (oracle/_ref/libgrisref.so for the GRIS pass, oracle/_ref/libdiref.so for ReSTIR DI).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's CPU legs import it.

Both libraries expose the same entry points (prefix `oracle_` / `gref_`); `run_sequence`
replays the renderer's frame loop (src/Renderer.cpp:329-347 ping-pong, 539-569 draw order):
G-buffer into slot j, GRISReSTIR::render with This = R[j], Prev = R[j^1], then j ^= 1.
All frame buffers start zeroed, as on the GPU side.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libgrisref.so")
DI_REF_LIB = os.path.join(HERE, "_ref", "libdiref.so")
POST_REF_LIB = os.path.join(HERE, "_ref", "libpostref.so")


class CpuImpl:
    def __init__(self, path, prefix):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        vp, u64 = ctypes.c_void_p, ctypes.c_ulonglong
        self._fn("scene_set", ctypes.c_int, [vp, u64] * 7)
        self._fn("gbuffer", None, [vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp])
        self._fn("gris_frame", None, [vp] * 12 + [ctypes.c_int])
        self._fn("counters", None, [vp, ctypes.c_int])
        self._fn("trace", None, [vp, u64, ctypes.c_int, vp, vp, vp])
        self._fn("sizeof", ctypes.c_int, [ctypes.c_int])
        self._fn("di_frame", None, [vp] * 12 + [ctypes.c_int], optional=True)
        self._arrays = None

    def _fn(self, name, res, args, optional=False):
        f = getattr(self.lib, self.prefix + name, None)
        if f is None and optional:
            setattr(self, name, None)
            return
        f.restype, f.argtypes = res, args
        setattr(self, name, f)

    def set_scene(self, host_scene):
        arrs = [np.ascontiguousarray(a) for a in host_scene.arrays()]
        self._arrays = arrs   # keep alive (the reference harness binds the arrays in place)
        args = []
        for a in arrs:
            args += [a.ctypes.data, len(a)]
        return self.scene_set(*args)

    def set_traversal(self, use_bvh):
        f = getattr(self.lib, self.prefix + "set_traversal", None)
        if f is not None:
            f.argtypes = [ctypes.c_int]
            f(int(use_bvh))

    def set_rows(self, y0, y1):
        f = self.lib.oracle_set_rows
        f.argtypes = [ctypes.c_int, ctypes.c_int]
        f(int(y0), int(y1))

    def select_scene(self, slot):
        """Makes scene slot `slot` current (the oracle keeps several scenes resident)."""
        f = self.lib.oracle_scene_select
        f.argtypes, f.restype = [ctypes.c_int], ctypes.c_int
        if f(int(slot)) != 0:
            raise ValueError("bad scene slot %d" % slot)

    def threads(self):
        return int(self.lib.oracle_threads())

    def read_counters(self, reset=True):
        out = (ctypes.c_ulonglong * 4)()
        self.counters(out, int(reset))
        return list(out)

    def trace_rays(self, rays, any_hit=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = len(rays)
        tuv = np.zeros((n, 4), np.float32)
        inst = np.zeros(n, np.uint32)
        tri = np.zeros(n, np.uint32)
        self.trace(rays.ctypes.data, n, int(any_hit), tuv.ctypes.data, inst.ctypes.data, tri.ctypes.data)
        return tuv, inst, tri


def oracle():
    return CpuImpl(ORACLE_LIB, "oracle_")


def reference():
    return CpuImpl(REF_LIB, "gref_")


class DiReference:
    """The reference's ReSTIR DI shaders compiled as C++ (oracle/_ref/libdiref.so): scene binding,
    ray counters and one TestReSTIR::render (dref_di_frame). No G-buffer of its own: the frames
    take the G-buffer of the GRIS harness or of the oracle (identical)."""

    def __init__(self, path=DI_REF_LIB):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        vp, u64 = ctypes.c_void_p, ctypes.c_ulonglong
        self.lib.dref_scene_set.argtypes, self.lib.dref_scene_set.restype = [vp, u64] * 7, ctypes.c_int
        self.lib.dref_di_frame.argtypes, self.lib.dref_di_frame.restype = [vp] * 12 + [ctypes.c_int], None
        self.lib.dref_counters.argtypes, self.lib.dref_counters.restype = [vp, ctypes.c_int], None
        self.lib.dref_sizeof.restype = ctypes.c_int
        self.di_frame = self.lib.dref_di_frame
        self._arrays = None

    def set_scene(self, host_scene):
        arrs = [np.ascontiguousarray(a) for a in host_scene.arrays()]
        self._arrays = arrs
        args = []
        for a in arrs:
            args += [a.ctypes.data, len(a)]
        return self.lib.dref_scene_set(*args)

    def read_counters(self, reset=True):
        out = (ctypes.c_ulonglong * 4)()
        self.lib.dref_counters(out, int(reset))
        return list(out)


def reference_di():
    return DiReference()


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def run_sequence(impl, cams, prevs, settings, width, height, frames=None, record=("resv", "temp", "out", "dn", "am", "mv")):
    """Runs len(cams) frames; returns a list of dicts of per-frame buffer copies."""
    from grisrt import RESERVOIR
    n = width * height
    dn = [np.zeros((n, 4), np.float32) for _ in range(2)]
    am = [np.zeros((n, 2), np.uint32) for _ in range(2)]
    mv = np.zeros((n, 2), np.uint16)
    resv = [np.zeros(n, RESERVOIR) for _ in range(2)]
    temp = np.zeros(n, RESERVOIR)
    out = np.zeros((n, 4), np.float32)
    sbytes = bytes(memoryview(settings))
    sbuf = np.frombuffer(sbytes, dtype=np.uint8).copy()
    results = []
    j = 0
    for f in range(len(cams)):
        cb = np.frombuffer(cams[f].tobytes(), np.uint8).copy()
        pb = np.frombuffer(prevs[f].tobytes(), np.uint8).copy()
        impl.gbuffer(_p(cb), width, height, _p(dn[j]), _p(am[j]), _p(mv))
        impl.gris_frame(_p(cb), _p(pb), _p(sbuf), _p(dn[j]), _p(dn[j ^ 1]), _p(am[j]), _p(am[j ^ 1]), _p(mv),
                        _p(resv[j]), _p(resv[j ^ 1]), _p(temp), _p(out), 7)
        rec = {}
        if "resv" in record:
            rec["resv"] = resv[j].copy()
        if "temp" in record:
            rec["temp"] = temp.copy()
        if "out" in record:
            rec["out"] = out.copy()
        if "dn" in record:
            rec["dn"] = dn[j].copy()
        if "am" in record:
            rec["am"] = am[j].copy()
        if "mv" in record:
            rec["mv"] = mv.copy()
        results.append(rec)
        j ^= 1
    return results


def post_process(W, H, direct, indirect, post_settings, reference=False):
    """The oracle's presentation pass: returns (float32 [H*W, 4] colour, uint8 [H*W, 4] RGBA).
    reference=True: the reference's own post_proc.frag compiled as C++ (oracle/_ref/libpostref.so)
    in its place, for the pin."""
    vp = ctypes.c_void_p
    if reference:
        if not os.path.exists(POST_REF_LIB):
            raise FileNotFoundError(POST_REF_LIB)
        lib = ctypes.CDLL(POST_REF_LIB)
        fn = lib.pref_post
    else:
        from . import build_oracle
        lib = ctypes.CDLL(build_oracle.build())
        fn = lib.oracle_post
    fn.argtypes = [ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp, vp, vp]
    fn.restype = None
    n = W * H
    z = np.zeros((n, 4), np.float32)
    d = np.ascontiguousarray(direct if direct is not None else z, np.float32)
    i = np.ascontiguousarray(indirect if indirect is not None else z, np.float32)
    sb = np.frombuffer(bytes(memoryview(post_settings)), np.uint32).copy()
    color = np.zeros((n, 4), np.float32)
    rgba = np.zeros((n, 4), np.uint8)
    fn(W, H, _p(d), _p(i), _p(sb), _p(color), _p(rgba))
    return color, rgba


def run_di_sequence(gbuffer_impl, di_impl, cams, prevs, di_settings, width, height, record=("resv", "temp", "out")):
    """Frames of TestReSTIR::render with the renderer's ping-pong (src/Renderer.cpp:339-341): the
    G-buffer (gbuffer_impl) into slot j, the DI pass with This = R[j], Prev = R[j^1], j ^= 1.
    di_settings: grisrt.DISettings. Returns per-frame copies of the recorded buffers."""
    from grisrt import DI_RESERVOIR
    n = width * height
    dn = [np.zeros((n, 4), np.float32) for _ in range(2)]
    am = [np.zeros((n, 2), np.uint32) for _ in range(2)]
    mv = np.zeros((n, 2), np.uint16)
    resv = [np.zeros(n, DI_RESERVOIR) for _ in range(2)]
    temp = np.zeros(n, DI_RESERVOIR)
    out = np.zeros((n, 4), np.float32)
    sbuf = np.frombuffer(bytes(memoryview(di_settings)), dtype=np.uint8).copy()
    results = []
    j = 0
    for f in range(len(cams)):
        cb = np.frombuffer(cams[f].tobytes(), np.uint8).copy()
        pb = np.frombuffer(prevs[f].tobytes(), np.uint8).copy()
        gbuffer_impl.gbuffer(_p(cb), width, height, _p(dn[j]), _p(am[j]), _p(mv))
        di_impl.di_frame(_p(cb), _p(pb), _p(sbuf), _p(dn[j]), _p(dn[j ^ 1]), _p(am[j]), _p(am[j ^ 1]), _p(mv),
                         _p(resv[j]), _p(resv[j ^ 1]), _p(temp), _p(out), 7)
        rec = {}
        if "resv" in record:
            rec["resv"] = resv[j].copy()
        if "temp" in record:
            rec["temp"] = temp.copy()
        if "out" in record:
            rec["out"] = out.copy()
        results.append(rec)
        j ^= 1
    return results


class ConvergedFP64:
    """The FP64 CPU oracle of the converged image (oracle/converged_fp64.cpp): per-pixel mean and
    variance over `spp` independent paths of estimator 0 (the GRIS candidate sum) or 1 (the full
    indirect illumination), from a G-buffer (dn: float32 [H*W, 4], am: uint32 [H*W, 2])."""

    def __init__(self):
        from . import build_oracle
        self.lib = ctypes.CDLL(build_oracle.build())
        vp, u64 = ctypes.c_void_p, ctypes.c_ulonglong
        self.lib.fp64_scene_set.argtypes = [vp, u64] * 7
        self.lib.fp64_scene_set.restype = ctypes.c_int
        self.lib.fp64_render.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, u64, u64, u64, ctypes.c_int, vp, vp]
        self.lib.fp64_render.restype = None

    def set_scene(self, host_scene):
        arrs = [np.ascontiguousarray(a) for a in host_scene.arrays()]
        args = []
        for a in arrs:
            args += [a.ctypes.data, len(a)]
        n = self.lib.fp64_scene_set(*args)
        if n < 0:
            raise ValueError("scene not supported by the FP64 oracle (%d)" % n)
        return n

    def render(self, cam, settings, W, H, dn, am, rect=None, spp=256, seed=1, estimator=0, spp_begin=0):
        """Returns (mean [h*w, 3], variance of one sample [h*w, 3]) over the rectangle
        (x0, y0, x1, y1) (default: the whole frame)."""
        x0, y0, x1, y1 = rect or (0, 0, W, H)
        n = (x1 - x0) * (y1 - y0)
        s = np.zeros((n, 3), np.float64)
        q = np.zeros((n, 3), np.float64)
        dn = np.ascontiguousarray(dn, np.float32)
        am = np.ascontiguousarray(am, np.uint32)
        cb = np.frombuffer(cam.tobytes(), np.uint8).copy()
        sb = np.frombuffer(bytes(memoryview(settings)), np.uint8).copy()
        self.lib.fp64_render(_p(cb), _p(sb), W, H, _p(dn), _p(am), x0, y0, x1, y1, spp_begin, spp, seed, estimator,
                             _p(s), _p(q))
        mean = s / spp
        var = np.maximum(q / spp - mean * mean, 0.0) * spp / max(1, spp - 1)
        return mean, var
