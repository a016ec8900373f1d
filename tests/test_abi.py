"""The C ABI boundary on a machine without a GPU: the libraries load, export
every function their public headers declare, and the ICD answers the loader
interface (negotiation, proc-address lookup, manifest) without a device."""
import ctypes
import json
import os
import re

import pytest

import cpvulkan_gb300 as c

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix_re):
    text = open(os.path.join(ROOT, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
    return sorted(set(re.findall(prefix_re, text)))


def test_icd_exports_every_declared_symbol(native):
    names = declared("include/cpvulkan_gb300.h", r"CPV_EXPORT[^;(]*?\b(\w+)\s*\(")
    assert "vk_icdGetInstanceProcAddr" in names and "cpv_queue_submit_no_alloc" in names
    lib = ctypes.CDLL(c.ICD_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_harness_exports_every_declared_symbol(native):
    names = declared("include/cpv_harness.h", r"\b(cpvh_\w+)\s*\(")
    assert len(names) >= 10
    lib = c.harness()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_exports_every_declared_symbol(oracle):
    names = declared("oracle/oracle.h", r"\b(cpv_oracle_\w+)\s*\(")
    missing = [n for n in names if not hasattr(oracle.lib, n)]
    assert not missing, missing


def test_loader_negotiation_and_proc_addr(native):
    lib = ctypes.CDLL(c.ICD_PATH)
    # The reference clamps the loader's version to 5 and keeps a lower one
    # (CPVulkan/CPVulkan.cpp:94-104).
    ver = ctypes.c_uint32(7)
    assert lib.vk_icdNegotiateLoaderICDInterfaceVersion(ctypes.byref(ver)) == 0
    assert ver.value == 5
    ver = ctypes.c_uint32(3)
    assert lib.vk_icdNegotiateLoaderICDInterfaceVersion(ctypes.byref(ver)) == 0
    assert ver.value == 3
    gipa = lib.vk_icdGetInstanceProcAddr
    gipa.restype = ctypes.c_void_p
    gipa.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    for name in (b"vkCreateInstance", b"vkEnumerateInstanceExtensionProperties", b"vkEnumerateInstanceVersion"):
        assert gipa(None, name), name
    assert not gipa(None, b"vkNotAFunction")
    gpa = lib.vk_icdGetPhysicalDeviceProcAddr
    gpa.restype = ctypes.c_void_p
    gpa.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    assert not gpa(None, b"vkGetPhysicalDeviceProperties")


def test_manifest_names_the_library(native):
    path = os.path.join(os.path.dirname(c.ICD_PATH), "CPVulkan.json")
    with open(path) as f:
        m = json.load(f)
    assert m["file_format_version"]
    lib = m["ICD"]["library_path"]
    lib = lib if os.path.isabs(lib) else os.path.join(os.path.dirname(path), lib)
    assert os.path.samefile(lib, c.ICD_PATH)
    assert m["ICD"]["api_version"].startswith("1.")


def test_diagnostics_without_device(native):
    lib = ctypes.CDLL(c.ICD_PATH)
    lib.cpv_last_error.restype = ctypes.c_char_p
    assert lib.cpv_last_error() is not None
    lib.cpv_kernel_launches.restype = ctypes.c_uint64
    assert lib.cpv_kernel_launches() >= 0
    assert lib.cpv_device_available() in (0, 1)


def test_no_alloc_submit_rejects_null(native):
    lib = ctypes.CDLL(c.ICD_PATH)
    f = lib.cpv_queue_submit_no_alloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    assert f(None, 0, None, None) != 0
    lib.cpv_last_error.restype = ctypes.c_char_p
    assert b"cpv_queue_submit_no_alloc" in lib.cpv_last_error()


def test_gpu_path_has_no_cpu_fallback(native):
    """Without a device, submissions fail loudly instead of rendering on the CPU."""
    if c.device_available():
        pytest.skip("a CUDA device is present")
    os.environ["CPV_COMPILE_ONLY"] = "1"
    try:
        ctx = c.Context()
        scene = c.Scene(c.CUBE, 1, [0])
        with pytest.raises(RuntimeError):
            r = c.Renderer(ctx, scene)
            r.render(1)
        ctx.close()
    finally:
        del os.environ["CPV_COMPILE_ONLY"]


def test_dynamic_state_commands_resolve(native):
    """Every vkCmdSet* of the reference's command buffer resolves (those for
    state a pipeline here never makes dynamic record nothing), so a loader's
    dispatch table has no null entry for them."""
    lib = ctypes.CDLL(c.ICD_PATH)
    gipa = lib.vk_icdGetInstanceProcAddr
    gipa.restype = ctypes.c_void_p
    gipa.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    instance = ctypes.c_void_p(16)  # the lookup does not dereference it
    for name in (b"vkCmdSetViewport", b"vkCmdSetScissor", b"vkCmdSetBlendConstants", b"vkCmdSetLineWidth", b"vkCmdSetDepthBias",
                 b"vkCmdSetDepthBounds", b"vkCmdSetStencilCompareMask", b"vkCmdSetStencilWriteMask", b"vkCmdSetStencilReference",
                 b"vkCmdCopyImage", b"vkCmdClearColorImage", b"vkCmdClearDepthStencilImage", b"vkCmdClearAttachments", b"vkCmdNextSubpass"):
        assert gipa(instance, name), name


def test_indirect_count_extension(native):
    """VK_KHR_draw_indirect_count and VK_AMD_draw_indirect_count are listed
    and their draw commands resolve under the reference's names
    (CPVulkan/Extensions.cpp:764-773, 1030-1038). Instance-level lookups take
    a non-null instance; the ICD's tables do not dereference it."""
    lib = ctypes.CDLL(c.ICD_PATH)
    gipa = lib.vk_icdGetInstanceProcAddr
    gipa.restype = ctypes.c_void_p
    gipa.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    instance = ctypes.c_void_p(16)
    for name in (b"vkCmdDrawIndirectCountKHR", b"vkCmdDrawIndexedIndirectCountKHR", b"vkCmdDrawIndirectCountAMD"):
        assert gipa(instance, name), name
    enum = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint32), ctypes.c_void_p)(
        gipa(instance, b"vkEnumerateDeviceExtensionProperties"))
    n = ctypes.c_uint32(0)
    assert enum(None, None, ctypes.byref(n), None) == 0 and n.value == 2

    class Props(ctypes.Structure):
        _fields_ = [("name", ctypes.c_char * 256), ("version", ctypes.c_uint32)]

    props = (Props * 2)()
    one = ctypes.c_uint32(1)
    assert enum(None, None, ctypes.byref(one), props) == 5 and one.value == 1  # VK_INCOMPLETE
    assert enum(None, None, ctypes.byref(n), props) == 0
    assert {(p.name, p.version) for p in props} == {(b"VK_KHR_draw_indirect_count", 1), (b"VK_AMD_draw_indirect_count", 2)}


def test_host_objects_use_the_application_allocator(native, monkeypatch):
    """Objects created with VkAllocationCallbacks live in the application's
    allocator and go back to it on destruction (the reference's Allocate /
    Free, CPVulkanBase/Base.h:256-294): one allocation and one free per
    object, none outstanding. Runs on the compile-only device."""
    monkeypatch.setenv("CPV_COMPILE_ONLY", "1")
    ctx = c.Context()
    try:
        objects, allocations, frees = ctx.allocator_check()
    finally:
        ctx.close()
    assert objects == 13
    assert allocations == objects and frees == allocations
