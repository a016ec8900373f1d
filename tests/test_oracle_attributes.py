"""The oracle's vertex attribute conversion (no GPU) against an independent
numpy restatement of the reference's rules, over every code: normalised
8/16-bit formats divide the integer by its type's maximum with no clamp of
the most negative signed code (LLVMRuntime/ImageCompiler.cpp:15-101,
161-230); half floats are widened exactly; B8G8R8A8 keeps red in byte 2;
absent components read 0, 0, 0, 1 (LLVMRuntime/PipelineCompiler.cpp:836-896)."""
import ctypes

import numpy as np
import pytest


def _decode(oracle, fmt, raw):
    lib = oracle.lib
    lib.cpv_oracle_decode_attribute.restype = ctypes.c_int
    lib.cpv_oracle_decode_attribute.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_float * 4)]
    out = (ctypes.c_float * 4)()
    buf = np.ascontiguousarray(np.frombuffer(bytes(raw) + b"\0" * 8, np.uint8))
    n = lib.cpv_oracle_decode_attribute(fmt, buf.ctypes.data, ctypes.byref(out))
    return n, np.array(out[:], np.float32)


def _bits(x):
    return np.asarray(x, np.float32).view(np.uint32)


@pytest.mark.parametrize("fmt,size,signed", [(9, 1, False), (10, 1, True), (70, 2, False), (71, 2, True)])
def test_normalised_every_code(oracle, fmt, size, signed):
    codes = np.arange(1 << (8 * size), dtype=np.int64)
    dt = {(1, False): np.uint8, (1, True): np.int8, (2, False): np.uint16, (2, True): np.int16}[(size, signed)]
    ints = codes.astype(np.uint64).astype(dt) if not signed else codes.astype(np.uint16 if size == 2 else np.uint8).view(dt)
    maxv = np.float32({(1, False): 255, (1, True): 127, (2, False): 65535, (2, True): 32767}[(size, signed)])
    want = ints.astype(np.float32) / maxv
    got = []
    for c in codes:
        n, out = _decode(oracle, fmt, int(c).to_bytes(size, "little"))
        assert n == 1
        assert out[1] == 0 and out[2] == 0 and out[3] == 1
        got.append(out[0])
    assert np.array_equal(_bits(got), _bits(want))
    if signed:
        assert got[1 << (8 * size - 1)] < -1.0  # the most negative code is not clamped


def test_half_every_code(oracle):
    codes = np.arange(1 << 16, dtype=np.uint32)
    want = codes.astype(np.uint16).view(np.float16).astype(np.float32)
    got = np.array([_decode(oracle, 76, int(c).to_bytes(2, "little"))[1][0] for c in codes], np.float32)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(_bits(got[~nan]), _bits(want[~nan]))


def test_channel_order_and_absent_components(oracle):
    n, out = _decode(oracle, 44, [10, 20, 30, 40])  # B8G8R8A8_UNORM
    assert n == 4 and np.array_equal(_bits(out), _bits(np.array([30, 20, 10, 40], np.float32) / np.float32(255)))
    n, out = _decode(oracle, 23, [255, 0, 51])      # R8G8B8_UNORM: alpha absent
    assert n == 3 and out[3] == 1.0 and out[0] == 1.0 and out[2] == np.float32(51) / np.float32(255)
    n, out = _decode(oracle, 78, [0xFF, 0x7F, 0x00, 0x80])  # R16G16_SNORM: 32767, -32768
    assert n == 2 and out[0] == 1.0 and out[1] == np.float32(-32768) / np.float32(32767) and out[2] == 0 and out[3] == 1
    n, out = _decode(oracle, 97, [0x00, 0x3C, 0x00, 0xC0, 0x01, 0x00, 0x00, 0x7C])  # 1, -2, smallest subnormal, +inf
    assert n == 4 and out[0] == 1.0 and out[1] == -2.0 and out[2] == np.float32(2.0 ** -24) and np.isinf(out[3])
    assert _decode(oracle, 98, [0, 0, 0, 0])[0] == -1  # R32_UINT is not a float attribute format here
