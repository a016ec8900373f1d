"""cpvulkan_gb300 — GB300 (sm_103a) Vulkan ICD for the draw hot path.

The product is the native library ``_build/libcpvulkan_gb300.so`` (a Vulkan
ICD loaded through ``_build/CPVulkan.json``). This module only locates and
builds the native libraries and wraps the headless harness
(``libcpv_harness.so``), which drives the ICD through Vulkan calls the way an
application behind the Vulkan loader does.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
ICD_PATH = os.path.join(BUILD_DIR, "libcpvulkan_gb300.so")
HARNESS_PATH = os.path.join(BUILD_DIR, "libcpv_harness.so")
MANIFEST_PATH = os.path.join(BUILD_DIR, "CPVulkan.json")

# Scene configurations (include/cpv_harness.h).
CUBE, HEIGHTFIELD, BLEND, BATCH, PROGRAM, SERVE = 1, 2, 3, 4, 5, 6
# Shader programs (include/cpv/scene.h).
(PROGRAM_CUBE, PROGRAM_TEXLIT, PROGRAM_FLATQUAD, PROGRAM_MESHPC, PROGRAM_DISCARD, PROGRAM_NOPERSP, PROGRAM_POINTS, PROGRAM_FETCH, PROGRAM_MRT,
 PROGRAM_MRTI, PROGRAM_STORAGE, PROGRAM_SEPARATE, PROGRAM_MATHX, PROGRAM_CALLS, PROGRAM_SSBO) = range(15)

VK_FORMAT_D16_UNORM = 124
VK_FORMAT_D32_SFLOAT = 126
VK_FORMAT_D32_SFLOAT_S8_UINT = 130
VK_SUCCESS = 0


def build():
    """Compiles the native libraries (nvcc/g++, sm_103a) if sources changed."""
    from . import native_build
    return native_build.build()


class SamplerDesc(ctypes.Structure):
    """cpv_scene_sampler (include/cpv/scene.h)."""
    _fields_ = [(n, ctypes.c_uint32) for n in ("mag_filter", "min_filter", "mipmap_mode", "address_u", "address_v", "address_w")] + \
               [(n, ctypes.c_float) for n in ("mip_lod_bias", "min_lod", "max_lod")] + [("border_color", ctypes.c_uint32)]


class SceneHeader(ctypes.Structure):
    """cpv_scene (include/cpv/scene.h)."""
    u32, f32, u64, vp = ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64, ctypes.c_void_p
    _fields_ = [("width", u32), ("height", u32), ("color_format", u32), ("depth_format", u32), ("clear_color", f32 * 4),
                ("clear_depth", f32), ("clear_stencil", u32), ("viewport", f32 * 6), ("vertex_data", vp), ("vertex_bytes", u64),
                ("index_data", vp), ("index_bytes", u64), ("index_type", u32), ("uniform_data", vp), ("uniform_bytes", u32),
                ("texture_data", vp), ("texture_bytes", u64), ("texture_width", u32), ("texture_height", u32),
                ("texture_levels", u32), ("texture_format", u32), ("sampler", SamplerDesc), ("num_pipelines", u32),
                ("pipelines", vp), ("num_draws", u32), ("draws", vp), ("extra_color_count", u32), ("extra_color_formats", u32 * 7),
                ("spec_lod", u32), ("texture_binding", u32), ("uniform_as_storage", u32)]


class SceneDraw(ctypes.Structure):
    """cpv_scene_draw (include/cpv/scene.h)."""
    u32 = ctypes.c_uint32
    _fields_ = [("pipeline", u32), ("indexed", u32), ("count", u32), ("instance_count", u32), ("first", u32),
                ("vertex_offset", ctypes.c_int32), ("first_instance", u32), ("push_size", u32),
                ("vertex_offsets", ctypes.c_uint64 * 4), ("index_offset", ctypes.c_uint64), ("push", ctypes.c_uint8 * 128)]


def depth_texel_bytes(fmt):
    return {0: 0, VK_FORMAT_D16_UNORM: 2, VK_FORMAT_D32_SFLOAT: 4, VK_FORMAT_D32_SFLOAT_S8_UINT: 8}[fmt]


def colour_texel_bytes(fmt):
    """Bytes per texel of a colour attachment format (R8_UNORM 1; R8G8_UNORM
    and R16_UNORM 2; the 4-byte formats otherwise); a depth-only pass reads
    back zeros in the 4-byte layout."""
    return {0: 4, 9: 1, 13: 1, 14: 1, 16: 2, 20: 2, 21: 2, 70: 2, 74: 2, 75: 2, 91: 8, 95: 8, 96: 8, 97: 8, 101: 8, 102: 8, 103: 8,
            107: 16, 108: 16, 109: 16}.get(fmt, 4)


_harness = None


def harness():
    """Loads libcpv_harness.so (building it first when missing)."""
    global _harness
    if _harness is not None:
        return _harness
    if not os.path.exists(HARNESS_PATH):
        build()
    h = ctypes.CDLL(HARNESS_PATH)
    vp, u32, u64, cp = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_char_p
    h.cpvh_scene_create.restype = vp
    h.cpvh_scene_create.argtypes = [u32, u64, ctypes.POINTER(u64), u32]
    h.cpvh_scene_destroy.argtypes = [vp]
    h.cpvh_scene_set_frame.argtypes = [vp, u32]
    h.cpvh_scene_triangles.restype = u64
    h.cpvh_scene_triangles.argtypes = [vp]
    h.cpvh_open.restype = vp
    h.cpvh_open.argtypes = [cp, cp, u32]
    h.cpvh_close.argtypes = [vp]
    h.cpvh_renderer_create.restype = vp
    h.cpvh_renderer_create.argtypes = [vp, vp, cp, u32]
    h.cpvh_renderer_destroy.argtypes = [vp]
    h.cpvh_compile_pipelines.restype = ctypes.c_int
    h.cpvh_compile_pipelines.argtypes = [vp, vp, cp, u32]
    h.cpvh_render.restype = ctypes.c_int
    h.cpvh_render.argtypes = [vp, u32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    h.cpvh_render_e2e.restype = ctypes.c_int
    h.cpvh_render_e2e.argtypes = [vp, u32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(u64), ctypes.POINTER(u64)]
    h.cpvh_renderer_update.restype = ctypes.c_int
    h.cpvh_renderer_update.argtypes = [vp]
    h.cpvh_renderer_set_indirect.restype = ctypes.c_int
    h.cpvh_renderer_set_indirect.argtypes = [vp, u32, vp]
    h.cpvh_renderer_set_indirect_count.restype = ctypes.c_int
    h.cpvh_renderer_set_indirect_count.argtypes = [vp, u32, u32]
    h.cpvh_readback.restype = ctypes.c_int
    h.cpvh_readback.argtypes = [vp, vp, vp]
    h.cpvh_readback_extra.restype = ctypes.c_int
    h.cpvh_readback_extra.argtypes = [vp, u32, vp]
    h.cpvh_queue.restype = vp
    h.cpvh_queue.argtypes = [vp]
    h.cpvh_last_error.restype = cp
    h.cpvh_allocator_check.restype = ctypes.c_int
    h.cpvh_allocator_check.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(u64)]
    h.cpvh_image_ops.restype = ctypes.c_int
    h.cpvh_image_ops.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, u32, vp, cp, u32]
    h.cpvh_blit.restype = ctypes.c_int
    h.cpvh_blit.argtypes = [vp, vp, u32, u32, u32, u32, vp, u32, u32, u32, u32, vp, u32, u32, cp, u32]
    h.cpvh_server_create.restype = vp
    h.cpvh_server_create.argtypes = [vp, ctypes.POINTER(ServeConfig), cp, u32]
    h.cpvh_server_run.restype = ctypes.c_int
    h.cpvh_server_run.argtypes = [vp, ctypes.POINTER(ServeResult)]
    h.cpvh_server_set_load.restype = None
    h.cpvh_server_set_load.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    h.cpvh_server_clients.restype = u32
    h.cpvh_server_clients.argtypes = [vp]
    h.cpvh_server_client.restype = vp
    h.cpvh_server_client.argtypes = [vp, u32]
    h.cpvh_server_scene.restype = vp
    h.cpvh_server_scene.argtypes = [vp, u32]
    h.cpvh_server_destroy.argtypes = [vp]
    _harness = h
    return h


class Scene:
    """A seeded scene owned by the harness (plain-data cpv_scene)."""

    def __init__(self, config, seed=1, params=()):
        h = harness()
        arr = (ctypes.c_uint64 * max(1, len(params)))(*[int(p) for p in params])
        self.ptr = h.cpvh_scene_create(config, seed, arr, len(params))
        if not self.ptr:
            raise ValueError("unknown scene configuration %r" % config)
        hdr = SceneHeader.from_address(self.ptr)
        self.width, self.height = hdr.width, hdr.height
        self.color_format, self.depth_format = hdr.color_format, hdr.depth_format
        # formats of the colour attachments after the first (0: unused reference)
        self.extra_color_formats = [hdr.extra_color_formats[k] for k in range(hdr.extra_color_count)]
        self.config = config

    @property
    def draws(self):
        return SceneHeader.from_address(self.ptr).num_draws

    @property
    def spec_lod(self):
        """1 when the oracle renders the scene in the quad-derivative LOD mode
        (the ICD's CPV_SPEC_LOD=1); 0 for the reference's λ = 0."""
        return SceneHeader.from_address(self.ptr).spec_lod

    @spec_lod.setter
    def spec_lod(self, value):
        SceneHeader.from_address(self.ptr).spec_lod = 1 if value else 0

    def draw(self, i):
        """Draw i of the scene (a view of the harness's cpv_scene_draw)."""
        h = SceneHeader.from_address(self.ptr)
        if not 0 <= i < h.num_draws:
            raise IndexError(i)
        return SceneDraw.from_address(h.draws + i * ctypes.sizeof(SceneDraw))

    def indirect_record(self, i):
        """Draw i as its VkDrawIndexedIndirectCommand / VkDrawIndirectCommand words."""
        d = self.draw(i)
        if d.indexed:
            return [d.count, d.instance_count, d.first, d.vertex_offset & 0xFFFFFFFF, d.first_instance]
        return [d.count, d.instance_count, d.first, d.first_instance, 0]

    @property
    def input_bytes(self):
        """Vertex, index, uniform and texture bytes of the scene."""
        h = SceneHeader.from_address(self.ptr)
        return h.vertex_bytes + h.index_bytes + h.uniform_bytes + h.texture_bytes

    @property
    def triangles(self):
        return harness().cpvh_scene_triangles(self.ptr)

    def set_frame(self, frame):
        harness().cpvh_scene_set_frame(self.ptr, frame)

    def close(self):
        if self.ptr:
            harness().cpvh_scene_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


OP_CLEAR_COLOR_IMAGE, OP_CLEAR_DEPTH_STENCIL_IMAGE, OP_COPY_IMAGE, OP_CLEAR_ATTACHMENTS = 0, 1, 2, 3


class ImageOp(ctypes.Structure):
    """cpvh_image_op (include/cpv_harness.h)."""
    u32, i32 = ctypes.c_uint32, ctypes.c_int32
    _fields_ = [("kind", u32), ("aspect", u32), ("level", u32), ("level_count", u32), ("src_level", u32), ("x", i32), ("y", i32),
                ("src_x", i32), ("src_y", i32), ("w", u32), ("h", u32), ("colour", ctypes.c_float * 4), ("depth", ctypes.c_float),
                ("stencil", u32)]


class Context:
    """An ICD loaded the loader's way, with one device and queue."""

    def __init__(self, icd_path=ICD_PATH):
        h = harness()
        err = ctypes.create_string_buffer(1024)
        self.ptr = h.cpvh_open(icd_path.encode(), err, len(err))
        if not self.ptr:
            raise RuntimeError("cannot open ICD: " + err.value.decode(errors="replace"))

    def compile_pipelines(self, scene):
        err = ctypes.create_string_buffer(4096)
        r = harness().cpvh_compile_pipelines(self.ptr, scene.ptr, err, len(err))
        if r != VK_SUCCESS:
            raise RuntimeError("pipeline compilation failed (%d): %s" % (r, err.value.decode(errors="replace")))

    def blit(self, src, src_size, src_levels, src_format, regions, filter, dst=None, dst_size=None, dst_levels=1,
             dst_format=None):
        """vkCmdBlitImage between RGBA8/BGRA8 images given as packed mip
        chains (uint8 numpy arrays). regions: sequence of
        (src_level, sx0, sy0, sx1, sy1, dst_level, dx0, dy0, dx1, dy1).
        Updates dst in place, or src when dst is None (blits within one
        image)."""
        import numpy as np

        reg = np.ascontiguousarray(np.asarray(regions, dtype=np.int32).reshape(-1, 10))
        err = ctypes.create_string_buffer(1024)
        dw, dh = dst_size if dst is not None else (0, 0)
        r = harness().cpvh_blit(self.ptr, src.ctypes.data, src_size[0], src_size[1], src_levels, src_format,
                                dst.ctypes.data if dst is not None else None, dw, dh, dst_levels,
                                dst_format if dst_format is not None else src_format, reg.ctypes.data, reg.shape[0],
                                filter, err, len(err))
        if r != VK_SUCCESS:
            raise RuntimeError("blit failed (%d): %s" % (r, err.value.decode(errors="replace")))

    def image_ops(self, format, size, levels, init0, ops, init1=None):
        """vkCmdClearColorImage / vkCmdClearDepthStencilImage /
        vkCmdCopyImage / vkCmdClearAttachments on image 0 of two images of
        `format` given as packed mip chains (uint8 numpy arrays in the ICD's
        texel layout); ops: dicts of ImageOp fields. Returns image 0's bytes."""
        import numpy as np

        arr = (ImageOp * max(1, len(ops)))()
        for i, op in enumerate(ops):
            for k, v in op.items():
                if k == "colour":
                    arr[i].colour[:] = list(v)
                else:
                    setattr(arr[i], k, v)
        init0 = np.ascontiguousarray(init0, dtype=np.uint8)
        init1 = None if init1 is None else np.ascontiguousarray(init1, dtype=np.uint8)
        out = np.zeros_like(init0)
        err = ctypes.create_string_buffer(1024)
        r = harness().cpvh_image_ops(self.ptr, format, size[0], size[1], levels, init0.ctypes.data,
                                     init1.ctypes.data if init1 is not None else None, arr, len(ops), out.ctypes.data, err, len(err))
        if r != VK_SUCCESS:
            raise RuntimeError("image ops failed (%d): %s" % (r, err.value.decode(errors="replace")))
        return out

    def allocator_check(self):
        """(objects, allocations, frees) of cpvh_allocator_check."""
        o, a, f = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
        r = harness().cpvh_allocator_check(self.ptr, ctypes.byref(o), ctypes.byref(a), ctypes.byref(f))
        if r != VK_SUCCESS:
            raise RuntimeError("allocator check failed (%d)" % r)
        return o.value, a.value, f.value

    @property
    def queue(self):
        return harness().cpvh_queue(self.ptr)

    def close(self):
        if self.ptr:
            harness().cpvh_close(self.ptr)
            self.ptr = None


class Renderer:
    """All Vulkan objects of one scene plus its recorded frame."""

    def __init__(self, ctx, scene):
        h = harness()
        err = ctypes.create_string_buffer(4096)
        self.scene = scene
        self.ctx = ctx
        self.ptr = h.cpvh_renderer_create(ctx.ptr, scene.ptr, err, len(err))
        if not self.ptr:
            raise RuntimeError("renderer creation failed: " + err.value.decode(errors="replace"))

    def render(self, frames=1, latencies=False):
        """Submits the frame `frames` times. Returns (device_ms, latencies_ms or None)."""
        dev = ctypes.c_double(0.0)
        lat = (ctypes.c_double * frames)() if latencies else None
        r = harness().cpvh_render(self.ptr, frames, ctypes.byref(dev), lat)
        if r != VK_SUCCESS:
            raise RuntimeError("render failed (%d): %s %s" % (r, harness().cpvh_last_error().decode(), icd_last_error()))
        return dev.value, (np.array(lat[:]) if latencies else None)

    def render_e2e(self, frames=1):
        total = ctypes.c_double(0.0)
        h2d, d2h = ctypes.c_uint64(0), ctypes.c_uint64(0)
        r = harness().cpvh_render_e2e(self.ptr, frames, ctypes.byref(total), ctypes.byref(h2d), ctypes.byref(d2h))
        if r != VK_SUCCESS:
            raise RuntimeError("end-to-end render failed (%d)" % r)
        return total.value, h2d.value, d2h.value

    def update(self):
        r = harness().cpvh_renderer_update(self.ptr)
        if r != VK_SUCCESS:
            raise RuntimeError("update failed (%d)" % r)

    def set_indirect(self, draw, record):
        """Overwrites draw `draw`'s indirect record (renderers created with
        CPVH_INDIRECT=1 or 2): [count, instances, first, vertex offset or first
        instance, first instance or 0]."""
        rec = (ctypes.c_uint32 * 5)(*[int(v) & 0xFFFFFFFF for v in (list(record) + [0] * 5)[:5]])
        r = harness().cpvh_renderer_set_indirect(self.ptr, draw, rec)
        if r != VK_SUCCESS:
            raise RuntimeError("set_indirect failed (%d)" % r)

    def set_indirect_count(self, draw, count):
        """Overwrites draw `draw`'s count word (renderers created with
        CPVH_INDIRECT=2, where each draw is an indirect-count draw of at most
        one record)."""
        r = harness().cpvh_renderer_set_indirect_count(self.ptr, draw, count)
        if r != VK_SUCCESS:
            raise RuntimeError("set_indirect_count failed (%d)" % r)

    def readback(self):
        s = self.scene
        color = np.zeros((s.height, s.width, colour_texel_bytes(s.color_format)), np.uint8)
        dsz = depth_texel_bytes(s.depth_format)
        depth = np.zeros((s.height, s.width, dsz), np.uint8) if dsz else None
        r = harness().cpvh_readback(self.ptr, color.ctypes.data, depth.ctypes.data if depth is not None else None)
        if r != VK_SUCCESS:
            raise RuntimeError("readback failed (%d)" % r)
        return color, depth

    def readback_extra(self, k):
        """Colour attachment k (1 .. 7) of the scene's subpass, as bytes per texel."""
        s = self.scene
        fmt = s.extra_color_formats[k - 1]
        out = np.zeros((s.height, s.width, colour_texel_bytes(fmt)), np.uint8)
        r = harness().cpvh_readback_extra(self.ptr, k, out.ctypes.data)
        if r != VK_SUCCESS:
            raise RuntimeError("readback of colour attachment %d failed (%d)" % (k, r))
        return out

    def close(self):
        if self.ptr and getattr(self, "owned", True):  # server client views belong to their server
            harness().cpvh_renderer_destroy(self.ptr)
        self.ptr = None


class ServeConfig(ctypes.Structure):
    """cpvh_serve_config (include/cpv_harness.h)."""
    _fields_ = [("clients", ctypes.c_uint32), ("slots", ctypes.c_uint32), ("mean_interarrival_ms", ctypes.c_double),
                ("duration_s", ctypes.c_double), ("seed", ctypes.c_uint64), ("hbm_budget_bytes", ctypes.c_uint64),
                ("min_tris", ctypes.c_uint32), ("max_tris", ctypes.c_uint32), ("max_side", ctypes.c_uint32),
                ("admit_on_demand", ctypes.c_uint32)]


class ServeResult(ctypes.Structure):
    """cpvh_serve_result (include/cpv_harness.h)."""
    _fields_ = [("requests", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("triangles", ctypes.c_uint64),
                ("resident_clients", ctypes.c_uint32), ("max_in_flight", ctypes.c_uint32), ("resident_bytes", ctypes.c_uint64),
                ("wall_s", ctypes.c_double), ("mtri_s", ctypes.c_double),
                ("latency_p50_ms", ctypes.c_double), ("latency_p99_ms", ctypes.c_double),
                ("submit_p50_ms", ctypes.c_double), ("submit_p99_ms", ctypes.c_double),
                ("queue_p50_ms", ctypes.c_double), ("queue_p99_ms", ctypes.c_double),
                ("residencies", ctypes.c_uint64), ("evictions", ctypes.c_uint64),
                ("residency_p50_ms", ctypes.c_double), ("residency_p99_ms", ctypes.c_double)]


class _ClientScene:
    """Dimensions of a server client's scene (for readback buffers)."""

    def __init__(self, ptr):
        hdr = SceneHeader.from_address(ptr)
        self.ptr = ptr
        self.width, self.height = hdr.width, hdr.height
        self.color_format, self.depth_format = hdr.color_format, hdr.depth_format


class Server:
    """Continuous-batching serving loop over resident offscreen clients."""

    def __init__(self, ctx, clients=64, slots=16, mean_interarrival_ms=2.0, duration_s=10.0, seed=5, hbm_budget_bytes=64 << 30,
                 min_tris=1000, max_tris=500000, max_side=0, admit_on_demand=True):
        cfg = ServeConfig(clients, slots, mean_interarrival_ms, duration_s, seed, hbm_budget_bytes, min_tris, max_tris, max_side,
                          1 if admit_on_demand else 0)
        self.ctx = ctx
        err = ctypes.create_string_buffer(4096)
        self.ptr = harness().cpvh_server_create(ctx.ptr, ctypes.byref(cfg), err, len(err))
        if not self.ptr:
            raise RuntimeError("server creation failed: " + err.value.decode(errors="replace"))

    @property
    def clients(self):
        return harness().cpvh_server_clients(self.ptr)

    def set_load(self, mean_interarrival_ms, duration_s):
        """Arrival rate and window of the next run (load sweeps)."""
        harness().cpvh_server_set_load(self.ptr, ctypes.c_double(mean_interarrival_ms), ctypes.c_double(duration_s))

    def run(self):
        res = ServeResult()
        r = harness().cpvh_server_run(self.ptr, ctypes.byref(res))
        if r != VK_SUCCESS:
            raise RuntimeError("serving loop failed (%d)" % r)
        return {k: getattr(res, k) for k, _ in ServeResult._fields_}

    def client(self, i):
        """A Renderer view of client i (readback, render alone)."""
        ptr = harness().cpvh_server_client(self.ptr, i)
        if not ptr:
            return None
        view = Renderer.__new__(Renderer)
        view.ptr = ptr
        view.ctx = None
        view.scene = _ClientScene(harness().cpvh_server_scene(self.ptr, i))
        view.owned = False
        return view

    def close(self):
        if self.ptr:
            harness().cpvh_server_destroy(self.ptr)
            self.ptr = None


def icd_last_error():
    """The ICD's last error message on this thread (cpv_last_error)."""
    lib = ctypes.CDLL(ICD_PATH)
    lib.cpv_last_error.restype = ctypes.c_char_p
    return lib.cpv_last_error().decode(errors="replace")


def batch_tuning():
    """The ICD's report of this thread's last batch tuning (cpv_batch_tuning)."""
    lib = ctypes.CDLL(ICD_PATH)
    lib.cpv_batch_tuning.restype = ctypes.c_char_p
    return lib.cpv_batch_tuning().decode(errors="replace")


def device_available():
    """True when the ICD can create a CUDA context (a GB300 is present)."""
    if not os.path.exists(ICD_PATH):
        build()
    lib = ctypes.CDLL(ICD_PATH)
    return bool(lib.cpv_device_available())


def kernel_launches():
    lib = ctypes.CDLL(ICD_PATH)
    lib.cpv_kernel_launches.restype = ctypes.c_uint64
    return lib.cpv_kernel_launches()
