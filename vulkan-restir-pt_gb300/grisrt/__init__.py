"""grisrt — Python bindings (ctypes) over the C ABI in include/grisrt.h.

The library is libgrisrt.so next to this file (built by vulkan-restir-pt_gb300/build.py).
There is no fallback: every GPU entry point goes to the CUDA kernels, and loading fails
loudly when the library is missing.

Numpy dtypes below are the reference's std430 layouts (src/shader/layouts.glsl), byte for
byte, so host arrays pass straight through the ABI.
"""
import ctypes
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# GRISRT_LIBRARY selects another build of the library (e.g. a variant being compared).
LIB_PATH = os.environ.get("GRISRT_LIBRARY") or os.path.join(_HERE, "libgrisrt.so")

# ---------------------------------------------------------------- layouts (numpy)
MATERIAL = np.dtype([("baseColor", "<f4", 3), ("type", "<u4"), ("textureIdx", "<u4"), ("metallic", "<f4"),
                     ("roughness", "<f4"), ("ior", "<f4")])
VERTEX = np.dtype([("pos", "<f4", 3), ("uvx", "<f4"), ("norm", "<f4", 3), ("uvy", "<f4")])
INSTANCE = np.dtype([("transform", "<f4", 16), ("transformInv", "<f4", 16), ("transformInvT", "<f4", 16),
                     ("radiance", "<f4", 3), ("pad0", "<f4"), ("indexOffset", "<u4"), ("indexCount", "<u4"),
                     ("matIndex", "<u4"), ("pad2", "<f4")])
LIGHT = np.dtype([("v0", "<f4", 3), ("nx", "<f4"), ("v1", "<f4", 3), ("ny", "<f4"), ("v2", "<f4", 3), ("nz", "<f4"),
                  ("radiance", "<f4", 3), ("area", "<f4")])
TABLE = np.dtype([("prob", "<f4"), ("failId", "<u4")])
RESERVOIR = np.dtype([("bary", "<f4", 2), ("instanceIdx", "<u4"), ("triangleIdx", "<u4"),
                      ("rcLi", "<f4", 3), ("rcRng", "<u4"), ("rcWi", "<f4", 3), ("flags", "<u4"),
                      ("pad", "<f4", 2), ("rcPrevSamplePdf", "<f4"), ("rcJacobian", "<f4"),
                      ("F", "<f4", 3), ("primaryRng", "<u4"),
                      ("sampleCount", "<f4"), ("resampleWeight", "<f4"), ("contribWeight", "<f4"), ("pad0", "<f4")])
# DIReservoir (layouts.glsl:96-115), 64 B; isLightSample is the GLSL bool as a 32-bit 0 / 1
DI_RESERVOIR = np.dtype([("bary", "<f4", 2), ("instanceIdx", "<u4"), ("triangleIdx", "<u4"),
                         ("Li", "<f4", 3), ("pad0", "<f4"), ("jacobian", "<f4"), ("samplePdf", "<f4"),
                         ("rng", "<u4"), ("isLightSample", "<u4"), ("sampleCount", "<u4"),
                         ("resampleWeight", "<f4"), ("contribWeight", "<f4"), ("weight", "<f4")])
assert DI_RESERVOIR.itemsize == 64
assert MATERIAL.itemsize == 32 and VERTEX.itemsize == 32 and INSTANCE.itemsize == 224
assert LIGHT.itemsize == 64 and TABLE.itemsize == 8 and RESERVOIR.itemsize == 96

INVALID_HIT = 0xFFFFFFFF
LAUNCH_GRID, LAUNCH_PERSISTENT = 0, 1
PATH_MEGAKERNEL, PATH_WAVEFRONT = 0, 1
NOALLOC_MAX_PIXELS = 65536
CLEAR_FLAG = 0x80000000
DI_SHIFT_RECONNECTION, DI_SHIFT_REPLAY, DI_SHIFT_HYBRID = 0, 1, 2
DI_SAMPLE_LIGHT, DI_SAMPLE_BSDF, DI_SAMPLE_BOTH = 0, 1, 2


class Camera(ctypes.Structure):
    """reference: Camera, layouts.glsl:27-51 (352 B)."""
    _fields_ = [("view", ctypes.c_float * 16), ("proj", ctypes.c_float * 16), ("projView", ctypes.c_float * 16),
                ("lastProjView", ctypes.c_float * 16), ("pos", ctypes.c_float * 3), ("FOV", ctypes.c_float),
                ("angle", ctypes.c_float * 3), ("nearZ", ctypes.c_float), ("front", ctypes.c_float * 3),
                ("farZ", ctypes.c_float), ("right", ctypes.c_float * 3), ("lensRadius", ctypes.c_float),
                ("up", ctypes.c_float * 3), ("focalDist", ctypes.c_float), ("filmSize", ctypes.c_uint32 * 2),
                ("frameIndex", ctypes.c_uint32), ("seed", ctypes.c_uint32)]

    def copy(self):
        c = Camera()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(Camera))
        return c

    def tobytes(self):
        return bytes(memoryview(self))


class Settings(ctypes.Structure):
    """GRISReSTIR::Settings (src/GRISReSTIR.h:11-17) + the reference's hard-coded constants."""
    _fields_ = [("shiftType", ctypes.c_uint32), ("rrScale", ctypes.c_float), ("temporalReuse", ctypes.c_uint32),
                ("spatialReuse", ctypes.c_uint32), ("cap", ctypes.c_uint32), ("maxDepth", ctypes.c_uint32),
                ("spatialNeighbors", ctypes.c_uint32), ("spatialRadius", ctypes.c_float),
                ("envRadiance", ctypes.c_float * 3), ("misWeights", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 4)]

    @classmethod
    def make(cls, shiftType=2, rrScale=1.0, temporalReuse=True, spatialReuse=True, cap=20, maxDepth=15,
             spatialNeighbors=3, spatialRadius=20.0, misWeights=0):
        s = cls()
        s.shiftType, s.rrScale, s.temporalReuse, s.spatialReuse = shiftType, rrScale, int(temporalReuse), int(spatialReuse)
        s.cap, s.maxDepth, s.spatialNeighbors, s.spatialRadius = cap, maxDepth, spatialNeighbors, spatialRadius
        s.misWeights = int(misWeights)
        return s


class DISettings(ctypes.Structure):
    """TestReSTIR::Settings (src/TestReSTIR.h:12-17); defaults as TestReSTIR.h:29."""
    _fields_ = [("shiftType", ctypes.c_uint32), ("sampleType", ctypes.c_uint32), ("temporalReuse", ctypes.c_uint32),
                ("spatialReuse", ctypes.c_uint32)]

    @classmethod
    def make(cls, shiftType=DI_SHIFT_RECONNECTION, sampleType=DI_SAMPLE_LIGHT, temporalReuse=False, spatialReuse=True):
        s = cls()
        s.shiftType, s.sampleType = shiftType, sampleType
        s.temporalReuse, s.spatialReuse = int(temporalReuse), int(spatialReuse)
        return s


class DIBindings(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("depthNormal", ctypes.c_void_p), ("depthNormalPrev", ctypes.c_void_p),
                ("albedoMatId", ctypes.c_void_p), ("albedoMatIdPrev", ctypes.c_void_p),
                ("motion", ctypes.c_void_p), ("reservoirThis", ctypes.c_void_p), ("reservoirPrev", ctypes.c_void_p),
                ("reservoirTemp", ctypes.c_void_p), ("directOutput", ctypes.c_void_p)]


TONEMAP_NONE, TONEMAP_FILMIC, TONEMAP_ACES = 0, 1, 2


class PostSettings(ctypes.Structure):
    """PostProcessFrag::PushConstant (src/PostProcessFrag.h:7-12); defaults as src/Renderer.h:32-33."""
    _fields_ = [("toneMapping", ctypes.c_uint32), ("correctGamma", ctypes.c_uint32), ("noDirect", ctypes.c_uint32),
                ("noIndirect", ctypes.c_uint32)]

    @classmethod
    def make(cls, toneMapping=TONEMAP_FILMIC, correctGamma=True, noDirect=False, noIndirect=False):
        s = cls()
        s.toneMapping, s.correctGamma = toneMapping, int(correctGamma)
        s.noDirect, s.noIndirect = int(noDirect), int(noIndirect)
        return s


class PostBindings(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("directOutput", ctypes.c_void_p),
                ("indirectOutput", ctypes.c_void_p), ("color", ctypes.c_void_p), ("rgba8", ctypes.c_void_p)]


def write_png(path, rgba, width, height):
    """8-bit RGBA pixels (uint8 [height*width, 4], row 0 at the top) into a PNG file (grisWritePNG)."""
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    if a.size != width * height * 4:
        raise ValueError("pixel array does not match %dx%d" % (width, height))
    err = ctypes.create_string_buffer(256)
    rc = load().grisWritePNG(os.fsencode(path), a.ctypes.data, width, height, err, 256)
    if rc != 0:
        raise GrisError("grisWritePNG failed (%d): %s" % (rc, err.value.decode(errors="replace")))


class SceneDesc(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_void_p), ("vertexCount", ctypes.c_uint64),
                ("indices", ctypes.c_void_p), ("indexCount", ctypes.c_uint64),
                ("instances", ctypes.c_void_p), ("instanceCount", ctypes.c_uint64),
                ("materials", ctypes.c_void_p), ("materialCount", ctypes.c_uint64),
                ("materialIndices", ctypes.c_void_p), ("materialIndexCount", ctypes.c_uint64),
                ("lights", ctypes.c_void_p), ("lightCount", ctypes.c_uint64),
                ("lightTable", ctypes.c_void_p), ("lightTableCount", ctypes.c_uint64)]


class PassBindings(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("depthNormal", ctypes.c_void_p), ("depthNormalPrev", ctypes.c_void_p),
                ("albedoMatId", ctypes.c_void_p), ("albedoMatIdPrev", ctypes.c_void_p),
                ("motion", ctypes.c_void_p), ("reservoirThis", ctypes.c_void_p), ("reservoirPrev", ctypes.c_void_p),
                ("reservoirTemp", ctypes.c_void_p), ("output", ctypes.c_void_p)]


class GBufferBindings(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("depthNormal", ctypes.c_void_p),
                ("albedoMatId", ctypes.c_void_p), ("motion", ctypes.c_void_p)]


class SceneStats(ctypes.Structure):
    _fields_ = [("triangleCount", ctypes.c_uint64), ("nodeCount", ctypes.c_uint64), ("nodeBytes", ctypes.c_uint64),
                ("triangleBytes", ctypes.c_uint64), ("maxDepth", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("buildSeconds", ctypes.c_double)]


class ConvergedBindings(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("depthNormal", ctypes.c_void_p),
                ("albedoMatId", ctypes.c_void_p), ("sum", ctypes.c_void_p), ("sumSq", ctypes.c_void_p)]


ESTIMATOR_CANDIDATES, ESTIMATOR_INDIRECT = 0, 1


class GuideConfig(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("learningRate", ctypes.c_float), ("mix", ctypes.c_float),
                ("samplesPerFrame", ctypes.c_uint32), ("stepsPerFrame", ctypes.c_uint32), ("train", ctypes.c_uint32),
                ("tensorCores", ctypes.c_uint32), ("trainKernel", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

    TRAIN_TCGEN05, TRAIN_MMA_SYNC = 0, 1

    @staticmethod
    def make(seed=1, learningRate=1e-3, mix=0.5, samplesPerFrame=1 << 18, stepsPerFrame=4, train=True, tensorCores=False,
             trainKernel=0):
        return GuideConfig(seed, learningRate, mix, samplesPerFrame, stepsPerFrame, int(train), int(tensorCores),
                           int(trainKernel))


class KernelProfile(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double), ("launches", ctypes.c_uint64), ("nodes", ctypes.c_uint64),
                ("tris", ctypes.c_uint64), ("rays", ctypes.c_uint64)]


PROFILE_SLOTS = ["gbuffer", "path_trace", "temporal", "spatial", "wave_begin", "wave_extend", "wave_shade",
                 "wave_shadow", "wave_post", "guide_infer", "guide_train", "di_candidates", "di_temporal",
                 "di_spatial", "reuse_vis_temporal", "reuse_vis_spatial"]


class TuneResult(ctypes.Structure):
    _fields_ = [("pathForm", ctypes.c_int), ("traceBlocksPerSM", ctypes.c_int), ("shadeBlocksPerSM", ctypes.c_int),
                ("candidates", ctypes.c_int), ("msPerFrame", ctypes.c_double), ("candidateMs", ctypes.c_double * 16),
                ("refill", ctypes.c_int)]


EXPORTS = [
    "grisCreate", "grisDestroy", "grisGetError", "grisSync", "grisGetStream", "grisReadCounters", "grisGetVersion",
    "grisSetProfiling", "grisReadProfile", "grisSetWorkCounting", "grisReadWorkCounters", "grisSetLaunchMode",
    "grisSizeof", "grisBuildLightTable", "grisCameraSetup", "grisCameraLookAt", "grisHostSceneCreate",
    "grisHostSceneDesc", "grisHostSceneCamera", "grisHostSceneDestroy", "grisSceneCreate", "grisSceneDestroy",
    "grisSceneGetStats", "grisDebugHostSceneCreate", "grisDebugTraceHost", "grisDebugTraceDevice", "grisPassGBuffer", "grisPassRender", "grisPassRenderNoAlloc",
    "grisNoAllocReadError", "grisMeasureL2Bandwidth",
    "grisFrameCreate", "grisFrameDestroy", "grisFrameRender", "grisFrameGetBuffer", "grisFrameDownload",
    "grisFrameUpload", "grisSetPathForm", "grisBatchCreate", "grisBatchDestroy", "grisBatchRender", "grisBatchGetBuffer",
    "grisBatchDownload", "grisFrameDownloadAsync", "grisBatchDownloadAsync", "grisDownloadWait", "grisSetGraphs", "grisSetWaveLaunch", "grisBatchAutotune",
    "grisReadKernelProfile", "grisConvergedAccumulate", "grisRelMSE",
    "grisGuideCreate", "grisGuideDestroy", "grisGuideParamCount", "grisGuideSetParams", "grisGuideGetParams",
    "grisGuideSetTraining", "grisGuideForward", "grisGuideGradient", "grisGuideTrainStep", "grisBatchSetGuide",
    "grisHostSceneLoad", "grisHostSceneFilmSize", "grisSetWaveRefill", "grisPassDI", "grisFrameRenderDI",
    "grisPostProcess", "grisWritePNG", "grisDebugGuideForwardStall",
]

_lib = None


def load(path=None):
    """Loads libgrisrt.so (raises if it is missing — there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libgrisrt.so not found at %s: run vulkan-restir-pt_gb300/build.py" % p)
    lib = ctypes.CDLL(p)
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    sig = {
        "grisCreate": (i32, [i32, ctypes.POINTER(vp)]),
        "grisDestroy": (i32, [vp]),
        "grisGetError": (ctypes.c_char_p, [vp]),
        "grisSync": (i32, [vp]),
        "grisGetStream": (vp, [vp]),
        "grisReadCounters": (i32, [vp, ctypes.POINTER(u64), i32]),
        "grisGetVersion": (i32, []),
        "grisSetProfiling": (i32, [vp, i32]),
        "grisReadProfile": (i32, [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(u64), i32]),
        "grisSetWorkCounting": (i32, [vp, i32]),
        "grisSetLaunchMode": (i32, [vp, i32]),
        "grisReadWorkCounters": (i32, [vp, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(u64), i32]),
        "grisSizeof": (ctypes.c_size_t, [i32]),
        "grisBuildLightTable": (i32, [vp, u32, vp]),
        "grisCameraSetup": (i32, [ctypes.POINTER(Camera), vp, vp, ctypes.c_float, u32, u32]),
        "grisCameraLookAt": (i32, [ctypes.POINTER(Camera), vp, vp, ctypes.c_float, u32, u32]),
        "grisHostSceneCreate": (i32, [i32, u64, u32, u32, ctypes.POINTER(vp)]),
        "grisHostSceneDesc": (i32, [vp, ctypes.POINTER(SceneDesc)]),
        "grisHostSceneCamera": (i32, [vp, u32, u32, u32, u32, ctypes.POINTER(Camera)]),
        "grisHostSceneDestroy": (i32, [vp]),
        "grisSceneCreate": (i32, [vp, ctypes.POINTER(SceneDesc), ctypes.POINTER(vp)]),
        "grisSceneDestroy": (i32, [vp]),
        "grisSceneGetStats": (i32, [vp, ctypes.POINTER(SceneStats)]),
        "grisDebugHostSceneCreate": (i32, [ctypes.POINTER(SceneDesc), ctypes.POINTER(vp)]),
        "grisDebugTraceHost": (i32, [vp, vp, u64, i32, vp, vp, vp]),
        "grisDebugTraceDevice": (i32, [vp, vp, vp, u64, i32, vp, vp, vp]),
        "grisPassGBuffer": (i32, [vp, vp, ctypes.POINTER(GBufferBindings), ctypes.POINTER(Camera)]),
        "grisPassRender": (i32, [vp, vp, ctypes.POINTER(PassBindings), ctypes.POINTER(Camera), ctypes.POINTER(Camera),
                                 ctypes.POINTER(Settings), i32]),
        "grisPassRenderNoAlloc": (i32, [vp, ctypes.POINTER(PassBindings), ctypes.POINTER(Camera), ctypes.POINTER(Camera),
                                        ctypes.POINTER(Settings), vp]),
        "grisNoAllocReadError": (i32, [i32, vp, ctypes.POINTER(u64)]),
        "grisMeasureL2Bandwidth": (i32, [vp, u64, i32, ctypes.POINTER(ctypes.c_double)]),
        "grisFrameCreate": (i32, [vp, u32, u32, ctypes.POINTER(vp)]),
        "grisFrameDestroy": (i32, [vp]),
        "grisFrameRender": (i32, [vp, vp, vp, ctypes.POINTER(Camera), ctypes.POINTER(Camera), ctypes.POINTER(Settings)]),
        "grisFrameGetBuffer": (i32, [vp, i32, i32, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t)]),
        "grisFrameDownload": (i32, [vp, vp, i32, i32, vp, ctypes.c_size_t]),
        "grisFrameUpload": (i32, [vp, vp, i32, i32, vp, ctypes.c_size_t]),
        "grisSetPathForm": (i32, [vp, i32]),
        "grisBatchCreate": (i32, [vp, u32, ctypes.POINTER(vp), ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(vp)]),
        "grisBatchDestroy": (i32, [vp]),
        "grisBatchRender": (i32, [vp, vp, ctypes.POINTER(Camera), ctypes.POINTER(Camera), ctypes.POINTER(Settings)]),
        "grisBatchGetBuffer": (i32, [vp, u32, i32, i32, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t)]),
        "grisBatchDownload": (i32, [vp, vp, u32, i32, i32, vp, ctypes.c_size_t]),
        "grisFrameDownloadAsync": (i32, [vp, vp, i32, i32, vp, ctypes.c_size_t]),
        "grisBatchDownloadAsync": (i32, [vp, vp, u32, i32, i32, vp, ctypes.c_size_t]),
        "grisDownloadWait": (i32, [vp]),
        "grisSetGraphs": (i32, [vp, i32]),
        "grisGuideCreate": (i32, [vp, ctypes.POINTER(GuideConfig), ctypes.POINTER(vp)]),
        "grisGuideDestroy": (i32, [vp]),
        "grisGuideParamCount": (i32, []),
        "grisGuideSetParams": (i32, [vp, vp, ctypes.c_size_t]),
        "grisGuideGetParams": (i32, [vp, vp, ctypes.c_size_t]),
        "grisGuideSetTraining": (i32, [vp, i32]),
        "grisGuideForward": (i32, [vp, vp, vp, u32, vp]),
        "grisDebugGuideForwardStall": (i32, [vp, vp, vp, u32, vp]),
        "grisGuideGradient": (i32, [vp, vp, vp, vp, vp, u32, vp]),
        "grisGuideTrainStep": (i32, [vp, vp, vp, vp, vp, u32]),
        "grisBatchSetGuide": (i32, [vp, vp]),
        "grisHostSceneLoad": (i32, [ctypes.c_char_p, ctypes.POINTER(vp), ctypes.c_char_p, ctypes.c_size_t]),
        "grisHostSceneFilmSize": (i32, [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]),
        "grisConvergedAccumulate": (i32, [vp, vp, ctypes.POINTER(ConvergedBindings), ctypes.POINTER(Camera),
                                          ctypes.POINTER(Settings), u32, u32, i32]),
        "grisRelMSE": (i32, [vp, vp, vp, ctypes.c_double, u64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
        "grisReadKernelProfile": (i32, [vp, ctypes.POINTER(KernelProfile), i32]),
        "grisSetWaveLaunch": (i32, [vp, i32, i32]),
        "grisSetWaveRefill": (i32, [vp, i32]),
        "grisPassDI": (i32, [vp, vp, ctypes.POINTER(DIBindings), ctypes.POINTER(Camera), ctypes.POINTER(Camera),
                             ctypes.POINTER(DISettings), i32]),
        "grisFrameRenderDI": (i32, [vp, vp, vp, ctypes.POINTER(Camera), ctypes.POINTER(Camera), ctypes.POINTER(Settings),
                                    ctypes.POINTER(DISettings)]),
        "grisPostProcess": (i32, [vp, ctypes.POINTER(PostBindings), ctypes.POINTER(PostSettings)]),
        "grisWritePNG": (i32, [ctypes.c_char_p, vp, u32, u32, ctypes.c_char_p, ctypes.c_size_t]),
        "grisBatchAutotune": (i32, [vp, vp, ctypes.POINTER(Camera), ctypes.POINTER(Camera), ctypes.POINTER(Settings), i32,
                                    ctypes.POINTER(TuneResult)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    _lib = lib
    return lib


class GrisError(RuntimeError):
    pass


def _check(rc, ctx=None, what=""):
    if rc != 0:
        msg = ""
        if ctx is not None:
            m = load().grisGetError(ctx)
            msg = m.decode() if m else ""
        raise GrisError("%s failed (%d): %s" % (what, rc, msg))


# ---------------------------------------------------------------- host helpers
def build_light_table(distribution):
    d = np.ascontiguousarray(distribution, dtype=np.float32)
    out = np.zeros(len(d) + 1, dtype=TABLE)
    _check(load().grisBuildLightTable(d.ctypes.data, len(d), out.ctypes.data), what="grisBuildLightTable")
    return out


def camera_setup(pos, angle, fov, width, height):
    c = Camera()
    p = np.asarray(pos, np.float32)
    a = np.asarray(angle, np.float32)
    _check(load().grisCameraSetup(ctypes.byref(c), p.ctypes.data, a.ctypes.data, fov, width, height), what="grisCameraSetup")
    return c


def scene_library(path):
    """Another build of the synthetic-scene generator (grisHostScene* and the camera helpers of
    csrc/host_scene.cpp) as a library of its own, for HostScene(lib=...): the CPU reference arm of
    the benchmark builds its inputs with it and loads no part of libgrisrt."""
    lib = ctypes.CDLL(path)
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    for name, (res, args) in {
            "grisHostSceneCreate": (i32, [i32, u64, u32, u32, ctypes.POINTER(vp)]),
            "grisHostSceneDesc": (i32, [vp, ctypes.POINTER(SceneDesc)]),
            "grisHostSceneCamera": (i32, [vp, u32, u32, u32, u32, ctypes.POINTER(Camera)]),
            "grisHostSceneDestroy": (i32, [vp])}.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    return lib


class HostScene:
    """Synthetic scene (kind 0 box, 1 terrain + spheres, 2 glossy terrain) as reference-layout arrays.
    lib: the library that generates it (default libgrisrt; see scene_library)."""

    def __init__(self, kind=0, seed=1, grid=512, spheres=2000, _handle=None, lib=None):
        lib = lib if lib is not None else load()
        self._lib = lib
        if _handle is None:
            h = ctypes.c_void_p()
            _check(lib.grisHostSceneCreate(kind, seed, grid, spheres, ctypes.byref(h)), what="grisHostSceneCreate")
        else:
            h = _handle
        self._h = h
        d = SceneDesc()
        _check(lib.grisHostSceneDesc(h, ctypes.byref(d)), what="grisHostSceneDesc")

        def arr(ptr, n, dt):
            if n == 0:
                return np.zeros(0, dtype=dt)
            buf = (ctypes.c_uint8 * (n * np.dtype(dt).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype=dt).copy()

        self.vertices = arr(d.vertices, d.vertexCount, VERTEX)
        self.indices = arr(d.indices, d.indexCount, np.uint32)
        self.instances = arr(d.instances, d.instanceCount, INSTANCE)
        self.materials = arr(d.materials, d.materialCount, MATERIAL)
        self.material_indices = arr(d.materialIndices, d.materialIndexCount, np.int32)
        self.lights = arr(d.lights, d.lightCount, LIGHT)
        self.light_table = arr(d.lightTable, d.lightTableCount, TABLE)

    @classmethod
    def load(cls, path):
        """A scene file in the reference's XML format with OBJ meshes (grisHostSceneLoad)."""
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = load().grisHostSceneLoad(os.fsencode(path), ctypes.byref(h), err, len(err))
        if rc != 0:
            raise GrisError("grisHostSceneLoad failed (%d): %s" % (rc, err.value.decode(errors="replace")))
        return cls(_handle=h)

    def film_size(self):
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        _check(load().grisHostSceneFilmSize(self._h, ctypes.byref(w), ctypes.byref(h)), what="grisHostSceneFilmSize")
        return w.value, h.value

    def camera(self, frame, frames, width, height):
        c = Camera()
        _check(self._lib.grisHostSceneCamera(self._h, frame, frames, width, height, ctypes.byref(c)),
               what="grisHostSceneCamera")
        return c

    def desc(self):
        d = SceneDesc()
        d.vertices, d.vertexCount = self.vertices.ctypes.data, len(self.vertices)
        d.indices, d.indexCount = self.indices.ctypes.data, len(self.indices)
        d.instances, d.instanceCount = self.instances.ctypes.data, len(self.instances)
        d.materials, d.materialCount = self.materials.ctypes.data, len(self.materials)
        d.materialIndices, d.materialIndexCount = self.material_indices.ctypes.data, len(self.material_indices)
        d.lights, d.lightCount = self.lights.ctypes.data, len(self.lights)
        d.lightTable, d.lightTableCount = self.light_table.ctypes.data, len(self.light_table)
        return d

    def arrays(self):
        return (self.vertices, self.indices, self.instances, self.materials, self.material_indices, self.lights,
                self.light_table)

    def triangle_count(self):
        return len(self.lights) + int(sum(int(i["indexCount"]) // 3 for i in self.instances))

    def __del__(self):
        lib = getattr(self, "_lib", None)
        if getattr(self, "_h", None) and lib is not None and not sys.is_finalizing():
            lib.grisHostSceneDestroy(self._h)
            self._h = None


def frame_seed(base, frame):
    """Per-frame camera seed (the reference draws it from std::default_random_engine in
    Camera::nextFrame, src/Camera.cpp:68-72; here a splitmix64 stream of the config seed)."""
    z = (int(base) * 0x9E3779B97F4A7C15 + (frame + 1) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return (z ^ (z >> 31)) >> 32


def sequence_cameras(host_scene, frames, width, height, seed=1, accumulate=False, orbit_frames=None):
    """Cameras of a frame sequence with the renderer's per-frame fields
    (src/Renderer.cpp:358-363, 654-660; src/Camera.cpp:68-98):
      seed         drawn per frame;
      frameIndex   clear flag on the first frame (no previous reservoirs), then 0 — or the
                   frame count when accumulating (running mean over frames);
      lastProjView the previous frame's projView (motion vectors);
      prev camera  the camera of the previous frame.
    Returns (cams, prevs)."""
    cams, prevs = [], []
    n = orbit_frames or frames
    for f in range(frames):
        c = host_scene.camera(f, n, width, height)
        c.seed = frame_seed(seed, f)
        if f > 0:
            ctypes.memmove(c.lastProjView, cams[f - 1].projView, 64)
        c.frameIndex = f if accumulate else (CLEAR_FLAG if f == 0 else 0)
        if accumulate and f == 0:
            c.frameIndex = CLEAR_FLAG
        cams.append(c)
        prevs.append(cams[f - 1].copy() if f > 0 else c.copy())
    return cams, prevs


# ---------------------------------------------------------------- device side
class Context:
    def __init__(self, device=0):
        lib = load()
        h = ctypes.c_void_p()
        _check(lib.grisCreate(device, ctypes.byref(h)), what="grisCreate")
        self.h = h

    def check(self, rc, what):
        _check(rc, self.h, what)

    def sync(self):
        self.check(load().grisSync(self.h), "grisSync")

    def stream(self):
        return load().grisGetStream(self.h)

    def download_wait(self):
        """Waits for the pipelined downloads queued so far (grisDownloadWait)."""
        self.check(load().grisDownloadWait(self.h), "grisDownloadWait")

    def l2_bandwidth(self, nbytes=48 << 20, reps=20):
        """L2 read bandwidth in GB/s (grisMeasureL2Bandwidth)."""
        g = ctypes.c_double()
        self.check(load().grisMeasureL2Bandwidth(self.h, int(nbytes), int(reps), ctypes.byref(g)), "grisMeasureL2Bandwidth")
        return g.value

    def counters(self, reset=False):
        out = (ctypes.c_uint64 * 4)()
        self.check(load().grisReadCounters(self.h, out, int(reset)), "grisReadCounters")
        return list(out)

    def set_profiling(self, enable):
        self.check(load().grisSetProfiling(self.h, int(enable)), "grisSetProfiling")

    def profile(self, reset=False):
        """(ms per kernel, launches per kernel) for G-buffer, path trace, temporal, spatial."""
        ms = (ctypes.c_double * 4)()
        n = (ctypes.c_uint64 * 4)()
        self.check(load().grisReadProfile(self.h, ms, n, int(reset)), "grisReadProfile")
        return list(ms), list(n)

    def post_process(self, bindings, post_settings):
        """grisPostProcess on device buffers (PostBindings of device pointers)."""
        self.check(load().grisPostProcess(self.h, ctypes.byref(bindings), ctypes.byref(post_settings)),
                   "grisPostProcess")

    def pass_di(self, scene, bindings, cam, prev_cam, di_settings, passes=7):
        """grisPassDI on caller buffers (DIBindings of device pointers)."""
        self.check(load().grisPassDI(self.h, scene.h, ctypes.byref(bindings), ctypes.byref(cam), ctypes.byref(prev_cam),
                                     ctypes.byref(di_settings), int(passes)), "grisPassDI")

    def kernel_profile(self, reset=False):
        """{slot name: dict(ms, launches, nodes, tris, rays)} over PROFILE_SLOTS."""
        out = (KernelProfile * len(PROFILE_SLOTS))()
        self.check(load().grisReadKernelProfile(self.h, out, int(reset)), "grisReadKernelProfile")
        return {name: dict(ms=o.ms, launches=o.launches, nodes=o.nodes, tris=o.tris, rays=o.rays)
                for name, o in zip(PROFILE_SLOTS, out)}

    def relmse(self, image_ptr, ref_sum_ptr, ref_scale, pixels, eps=1e-2):
        """(relMSE, MSE) of an RGBA32F device image against ref_sum * ref_scale (device FP64)."""
        out = (ctypes.c_double * 2)()
        self.check(load().grisRelMSE(self.h, ctypes.c_void_p(image_ptr), ctypes.c_void_p(ref_sum_ptr), float(ref_scale),
                                     int(pixels), float(eps), out), "grisRelMSE")
        return out[0], out[1]

    def set_launch_mode(self, mode):
        """0: grid (one thread per pixel, default), 1: persistent with per-lane refill."""
        self.check(load().grisSetLaunchMode(self.h, int(mode)), "grisSetLaunchMode")

    def set_path_form(self, form):
        """0: megakernel path tracer, 1: wavefront stages with per-bounce queues (batches)."""
        self.check(load().grisSetPathForm(self.h, int(form)), "grisSetPathForm")

    def set_graphs(self, enable):
        """Batch frames replay a captured CUDA graph (default on; off while profiling)."""
        self.check(load().grisSetGraphs(self.h, int(enable)), "grisSetGraphs")

    def set_wave_launch(self, trace_blocks_per_sm, shade_blocks_per_sm):
        self.check(load().grisSetWaveLaunch(self.h, int(trace_blocks_per_sm), int(shade_blocks_per_sm)),
                   "grisSetWaveLaunch")

    def set_wave_refill(self, enable):
        self.check(load().grisSetWaveRefill(self.h, int(enable)), "grisSetWaveRefill")

    def set_work_counting(self, enable):
        self.check(load().grisSetWorkCounting(self.h, int(enable)), "grisSetWorkCounting")

    def work(self, reset=False):
        """(nodes, triangles, closest-hit rays) per kernel."""
        a, b, c = (ctypes.c_uint64 * 4)(), (ctypes.c_uint64 * 4)(), (ctypes.c_uint64 * 4)()
        self.check(load().grisReadWorkCounters(self.h, a, b, c, int(reset)), "grisReadWorkCounters")
        return list(a), list(b), list(c)

    def close(self):
        if self.h:
            load().grisDestroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down: leave it to the driver
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class Scene:
    def __init__(self, ctx, host_scene):
        self.ctx = ctx
        self.host = host_scene
        self._desc = host_scene.desc()
        h = ctypes.c_void_p()
        ctx.check(load().grisSceneCreate(ctx.h, ctypes.byref(self._desc), ctypes.byref(h)), "grisSceneCreate")
        self.h = h

    def stats(self):
        s = SceneStats()
        self.ctx.check(load().grisSceneGetStats(self.h, ctypes.byref(s)), "grisSceneGetStats")
        return s

    def converged(self, cam, settings, width, height, depth_normal, albedo_matid, sum_ptr, sumsq_ptr=None,
                  spp_begin=0, spp=1, estimator=ESTIMATOR_CANDIDATES):
        """Adds `spp` samples per pixel of the converged-image estimator to the FP64 device sums
        (grisConvergedAccumulate); depth_normal / albedo_matid: the G-buffer of `cam`."""
        b = ConvergedBindings(width, height, depth_normal, albedo_matid, sum_ptr, sumsq_ptr)
        self.ctx.check(load().grisConvergedAccumulate(self.ctx.h, self.h, ctypes.byref(b), ctypes.byref(cam),
                                                      ctypes.byref(settings), int(spp_begin), int(spp), int(estimator)),
                       "grisConvergedAccumulate")

    def trace_host(self, rays, any_hit=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = len(rays)
        tuv = np.zeros((n, 4), np.float32)
        inst = np.zeros(n, np.uint32)
        tri = np.zeros(n, np.uint32)
        rc = load().grisDebugTraceHost(self.h, rays.ctypes.data, n, int(any_hit), tuv.ctypes.data, inst.ctypes.data,
                                       tri.ctypes.data)
        _check(rc, what="grisDebugTraceHost")
        return tuv, inst, tri

    def close(self):
        if self.h:
            if self.ctx.h:   # a context destroyed first (garbage collection order) took its objects' use with it
                load().grisSceneDestroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down: leave it to the driver
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


BUF_DEPTH_NORMAL, BUF_ALBEDO_MATID, BUF_MOTION, BUF_RESERVOIR, BUF_TEMP, BUF_OUTPUT = range(6)
BATCH_ALL_VIEWS = 0xFFFFFFFF   # a batch buffer of every view at once, in view order
BUF_DI_RESERVOIR, BUF_DI_TEMP, BUF_DIRECT_OUTPUT = 6, 7, 8
_BUF_DTYPE = {0: (np.float32, 4), 1: (np.uint32, 2), 2: (np.uint16, 2), 3: (RESERVOIR, None),
              4: (RESERVOIR, None), 5: (np.float32, 4), 6: (DI_RESERVOIR, None), 7: (DI_RESERVOIR, None),
              8: (np.float32, 4)}


class Frame:
    """Library-owned frame resources with the renderer's ping-pong (grisFrame*)."""

    def __init__(self, ctx, width, height):
        self.ctx, self.w, self.h = ctx, width, height
        h = ctypes.c_void_p()
        ctx.check(load().grisFrameCreate(ctx.h, width, height, ctypes.byref(h)), "grisFrameCreate")
        self.handle = h

    def render(self, scene, cam, prev_cam, settings):
        self.ctx.check(load().grisFrameRender(self.ctx.h, scene.h, self.handle, ctypes.byref(cam), ctypes.byref(prev_cam),
                                              ctypes.byref(settings)), "grisFrameRender")

    def render_di(self, scene, cam, prev_cam, di_settings, settings=None):
        """The renderer's frame with the ReSTIR DI pass (grisFrameRenderDI); settings=None skips the
        GRIS pass (indirect method None)."""
        self.ctx.check(load().grisFrameRenderDI(self.ctx.h, scene.h, self.handle, ctypes.byref(cam),
                                                ctypes.byref(prev_cam),
                                                ctypes.byref(settings) if settings is not None else None,
                                                ctypes.byref(di_settings)), "grisFrameRenderDI")

    def device_ptr(self, which, slot=0):
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        self.ctx.check(load().grisFrameGetBuffer(self.handle, which, slot, ctypes.byref(p), ctypes.byref(n)),
                       "grisFrameGetBuffer")
        return p.value, n.value

    def download(self, which, slot=0):
        dt, ch = _BUF_DTYPE[which]
        n = self.w * self.h
        arr = np.zeros((n, ch) if ch else n, dtype=dt)
        self.ctx.check(load().grisFrameDownload(self.ctx.h, self.handle, which, slot, arr.ctypes.data, arr.nbytes),
                       "grisFrameDownload")
        return arr

    def download_async(self, which, out, slot=0):
        """Queues a pipelined copy into the caller's host buffer `out` = (pointer, bytes); complete
        after Context.download_wait() (grisFrameDownloadAsync)."""
        ptr, nbytes = out
        self.ctx.check(load().grisFrameDownloadAsync(self.ctx.h, self.handle, which, slot, ctypes.c_void_p(ptr), nbytes),
                       "grisFrameDownloadAsync")

    def close(self):
        if self.handle:
            if self.ctx.h:   # a context destroyed first (garbage collection order) took its objects' use with it
                load().grisFrameDestroy(self.handle)
            self.handle = None

    def __del__(self):
        # at interpreter exit the CUDA runtime may already be torn down: leave it to the driver
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class Guide:
    """The guiding network (grisGuide*): parameters as one flat FP32 vector W0 b0 ... W4 b4
    (W row-major out x in), device-pointer forward / gradient / Adam step."""

    def __init__(self, ctx, config=None):
        self.ctx = ctx
        cfg = config or GuideConfig.make()
        h = ctypes.c_void_p()
        ctx.check(load().grisGuideCreate(ctx.h, ctypes.byref(cfg), ctypes.byref(h)), "grisGuideCreate")
        self.h = h
        self.n_params = load().grisGuideParamCount()

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        self.ctx.check(load().grisGuideGetParams(self.h, ctypes.c_void_p(p.ctypes.data), p.size), "grisGuideGetParams")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self.ctx.check(load().grisGuideSetParams(self.h, ctypes.c_void_p(p.ctypes.data), p.size), "grisGuideSetParams")

    def set_training(self, enable):
        self.ctx.check(load().grisGuideSetTraining(self.h, int(enable)), "grisGuideSetTraining")

    def forward(self, feat_ptr, n, out_ptr):
        self.ctx.check(load().grisGuideForward(self.ctx.h, self.h, ctypes.c_void_p(feat_ptr), n, ctypes.c_void_p(out_ptr)),
                       "grisGuideForward")

    def gradient(self, feat_ptr, dir_ptr, weight_ptr, n, grad_ptr):
        self.ctx.check(load().grisGuideGradient(self.ctx.h, self.h, ctypes.c_void_p(feat_ptr), ctypes.c_void_p(dir_ptr),
                                                ctypes.c_void_p(weight_ptr), n, ctypes.c_void_p(grad_ptr)),
                       "grisGuideGradient")

    def train_step(self, feat_ptr, dir_ptr, weight_ptr, n):
        self.ctx.check(load().grisGuideTrainStep(self.ctx.h, self.h, ctypes.c_void_p(feat_ptr), ctypes.c_void_p(dir_ptr),
                                                 ctypes.c_void_p(weight_ptr), n), "grisGuideTrainStep")

    def close(self):
        if self.h:
            if self.ctx.h:   # a context destroyed first (garbage collection order) took its objects' use with it
                load().grisGuideDestroy(self.h)
            self.h = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many views (own scene, size, cameras, settings) rendered with one launch per pass (grisBatch*)."""

    def __init__(self, ctx, scenes, sizes):
        self.ctx = ctx
        self.scenes = list(scenes)
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        n = len(self.scenes)
        sh = (ctypes.c_void_p * n)(*[sc.h.value for sc in self.scenes])
        ws = (ctypes.c_uint32 * n)(*[w for w, _ in self.sizes])
        hs = (ctypes.c_uint32 * n)(*[h for _, h in self.sizes])
        h = ctypes.c_void_p()
        ctx.check(load().grisBatchCreate(ctx.h, n, sh, ws, hs, ctypes.byref(h)), "grisBatchCreate")
        self.handle = h

    def render(self, cams, prev_cams, settings):
        n = len(self.scenes)
        c = (Camera * n)(*cams)
        p = (Camera * n)(*prev_cams)
        s = (Settings * n)(*settings)
        self.ctx.check(load().grisBatchRender(self.ctx.h, self.handle, c, p, s), "grisBatchRender")

    def set_guide(self, guide):
        """Attaches a Guide (None detaches): guided path sampling, and training if the guide trains."""
        self.guide = guide
        self.ctx.check(load().grisBatchSetGuide(self.handle, guide.h if guide is not None else None), "grisBatchSetGuide")

    def autotune(self, cams, prev_cams, settings, frames=3):
        """Times the candidate launch configurations on these views (rendering frames), keeps the
        fastest in the context and returns the TuneResult."""
        n = len(self.scenes)
        c = (Camera * n)(*cams)
        p = (Camera * n)(*prev_cams)
        s = (Settings * n)(*settings)
        r = TuneResult()
        self.ctx.check(load().grisBatchAutotune(self.ctx.h, self.handle, c, p, s, int(frames), ctypes.byref(r)),
                       "grisBatchAutotune")
        return r

    def device_ptr(self, view, which, slot=0):
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        self.ctx.check(load().grisBatchGetBuffer(self.handle, view, which, slot, ctypes.byref(p), ctypes.byref(n)),
                       "grisBatchGetBuffer")
        return p.value, n.value

    def download(self, view, which, slot=0, out=None):
        """Copies one view's buffer to the host (waits on the context stream)."""
        dt, ch = _BUF_DTYPE[which]
        px = sum(w * h for (w, h) in self.sizes) if view == BATCH_ALL_VIEWS else self.sizes[view][0] * self.sizes[view][1]
        if out is None:
            out = np.zeros((px, ch) if ch else px, dtype=dt)
            ptr, nbytes = out.ctypes.data, out.nbytes
        else:   # caller-provided host buffer (e.g. pinned): (pointer, bytes)
            ptr, nbytes = out
        self.ctx.check(load().grisBatchDownload(self.ctx.h, self.handle, view, which, slot, ctypes.c_void_p(ptr), nbytes),
                       "grisBatchDownload")
        return out

    def download_async(self, view, which, out, slot=0):
        """Queues a pipelined copy of one view's buffer into the caller's host buffer `out` =
        (pointer, bytes), pinned for the copy to overlap the next frame; complete after
        Context.download_wait() (grisBatchDownloadAsync)."""
        ptr, nbytes = out
        self.ctx.check(load().grisBatchDownloadAsync(self.ctx.h, self.handle, view, which, slot, ctypes.c_void_p(ptr),
                                                     nbytes), "grisBatchDownloadAsync")

    def close(self):
        if self.handle:
            if self.ctx.h:   # a context destroyed first (garbage collection order) took its objects' use with it
                load().grisBatchDestroy(self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass
