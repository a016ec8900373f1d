"""ctypes binding of the CPU oracle (oracle/), used only as the checker."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")


class Stats(ctypes.Structure):
    _fields_ = [("triangles", ctypes.c_uint64), ("vs_invocations", ctypes.c_uint64), ("fragments", ctypes.c_uint64),
                ("fragments_written", ctypes.c_uint64)]


class SamplerDesc(ctypes.Structure):
    _fields_ = [("mag_filter", ctypes.c_uint32), ("min_filter", ctypes.c_uint32), ("mipmap_mode", ctypes.c_uint32),
                ("address_u", ctypes.c_uint32), ("address_v", ctypes.c_uint32), ("address_w", ctypes.c_uint32),
                ("mip_lod_bias", ctypes.c_float), ("min_lod", ctypes.c_float), ("max_lod", ctypes.c_float),
                ("border_color", ctypes.c_uint32)]


class Oracle:
    def __init__(self, lib):
        self.lib = lib
        f, u32, vp = ctypes.c_float, ctypes.c_uint32, ctypes.c_void_p
        lib.cpv_oracle_render.restype = ctypes.c_int
        lib.cpv_oracle_render.argtypes = [vp, vp, vp, u32, u32, u32, ctypes.POINTER(Stats)]
        lib.cpv_oracle_render_extra.restype = ctypes.c_int
        lib.cpv_oracle_render_extra.argtypes = [vp, vp, vp, vp, u32, u32, u32, ctypes.POINTER(Stats)]
        lib.cpv_oracle_render_threaded.restype = ctypes.c_int
        lib.cpv_oracle_render_threaded.argtypes = [vp, vp, vp, u32, u32, u32, u32, ctypes.POINTER(Stats)]
        lib.cpv_oracle_edge.restype = f
        lib.cpv_oracle_edge.argtypes = [f] * 6
        lib.cpv_oracle_encode_unorm8.restype = ctypes.c_uint8
        lib.cpv_oracle_encode_unorm8.argtypes = [f]
        lib.cpv_oracle_encode_unorm16.restype = ctypes.c_uint16
        lib.cpv_oracle_encode_unorm16.argtypes = [f]
        lib.cpv_oracle_decode_unorm8.restype = f
        lib.cpv_oracle_decode_unorm8.argtypes = [ctypes.c_uint8]
        lib.cpv_oracle_logic_op.restype = ctypes.c_uint8
        lib.cpv_oracle_logic_op.argtypes = [ctypes.c_uint32, ctypes.c_uint8, ctypes.c_uint8]
        lib.cpv_oracle_sample.argtypes = [vp, u32, u32, u32, ctypes.POINTER(SamplerDesc), f, f, f, ctypes.POINTER(f * 4)]
        lib.cpv_oracle_blend.argtypes = [ctypes.POINTER(f * 4)] * 3 + [u32] * 6 + [ctypes.POINTER(f * 4)]
        lib.cpv_oracle_blit.argtypes = [vp, u32, u32, u32, vp, u32, u32, u32, vp, u32]

    def blit(self, src, src_format, dst, dst_format, region, filter):
        """One blit region between single levels (HxWx4 uint8 arrays, dst
        updated in place); region = (sx0, sy0, sx1, sy1, dx0, dy0, dx1, dy1)."""
        assert src.flags.c_contiguous and dst.flags.c_contiguous
        reg = np.ascontiguousarray(np.asarray(region, dtype=np.int32))
        self.lib.cpv_oracle_blit(src.ctypes.data, src.shape[1], src.shape[0], src_format, dst.ctypes.data, dst.shape[1],
                                 dst.shape[0], dst_format, reg.ctypes.data, filter)

    def render(self, scene, draw_begin=0, draw_end=None, color=None, depth=None, clear=True):
        """Renders a cpvulkan_gb300.Scene; returns (color HxWx4 u8, depth HxWxB u8 or None, stats dict)."""
        from cpvulkan_gb300 import colour_texel_bytes, depth_texel_bytes
        h, w = scene.height, scene.width
        dsz = depth_texel_bytes(scene.depth_format)
        color = np.zeros((h, w, colour_texel_bytes(scene.color_format)), np.uint8) if color is None else color
        if dsz and depth is None:
            depth = np.zeros((h, w, dsz), np.uint8)
        st = Stats()
        end = 0xFFFFFFFF if draw_end is None else draw_end
        r = self.lib.cpv_oracle_render(scene.ptr, color.ctypes.data, depth.ctypes.data if dsz else None, 1 if clear else 0,
                                       draw_begin, end, ctypes.byref(st))
        if r != 0:
            raise RuntimeError("oracle rejected the scene (%d)" % r)
        return color, (depth if dsz else None), {k: getattr(st, k) for k, _ in Stats._fields_}


    def render_extra(self, scene):
        """Renders a scene with colour attachments after the first; returns
        (color, [attachment 1, ...], depth or None, stats), each attachment
        HxWxB uint8 in its format (zeros for an unused reference)."""
        from cpvulkan_gb300 import colour_texel_bytes, depth_texel_bytes
        h, w = scene.height, scene.width
        color = np.zeros((h, w, colour_texel_bytes(scene.color_format)), np.uint8)
        extras = [np.zeros((h, w, colour_texel_bytes(f)), np.uint8) for f in scene.extra_color_formats]
        ptrs = (ctypes.c_void_p * 7)(*[(e.ctypes.data if f else None) for e, f in zip(extras, scene.extra_color_formats)])
        dsz = depth_texel_bytes(scene.depth_format)
        depth = np.zeros((h, w, dsz), np.uint8) if dsz else None
        st = Stats()
        r = self.lib.cpv_oracle_render_extra(scene.ptr, color.ctypes.data, ptrs, depth.ctypes.data if dsz else None, 1, 0, 0xFFFFFFFF,
                                             ctypes.byref(st))
        if r != 0:
            raise RuntimeError("oracle rejected the scene (%d)" % r)
        return color, extras, depth, {k: getattr(st, k) for k, _ in Stats._fields_}

    def render_threaded(self, scene, threads=None, draw_begin=0, draw_end=None, color=None, depth=None, clear=True):
        """render() on `threads` host threads (default: every usable core);
        the image is identical to render()'s."""
        from cpvulkan_gb300 import colour_texel_bytes, depth_texel_bytes
        if threads is None:
            threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        h, w = scene.height, scene.width
        dsz = depth_texel_bytes(scene.depth_format)
        color = np.zeros((h, w, colour_texel_bytes(scene.color_format)), np.uint8) if color is None else color
        if dsz and depth is None:
            depth = np.zeros((h, w, dsz), np.uint8)
        st = Stats()
        end = 0xFFFFFFFF if draw_end is None else draw_end
        r = self.lib.cpv_oracle_render_threaded(scene.ptr, color.ctypes.data, depth.ctypes.data if dsz else None, 1 if clear else 0,
                                                draw_begin, end, threads, ctypes.byref(st))
        if r != 0:
            raise RuntimeError("oracle rejected the scene (%d)" % r)
        return color, (depth if dsz else None), {k: getattr(st, k) for k, _ in Stats._fields_}


def build():
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR], stdout=subprocess.DEVNULL)


def load():
    build()
    return Oracle(ctypes.CDLL(LIB))
