"""Builds the native libraries of cpvulkan_gb300 in-tree (cpvulkan_gb300/_build).

* libcpvulkan_gb300.so — the Vulkan ICD: SPIR-V translator, NVRTC pipeline
  compiler, CUDA runtime layer (nvcc, sm_103a) and the Vulkan entry points.
* libcpv_harness.so   — the headless loader/application and scene generators.

The device headers used by NVRTC at pipeline creation and the SPIR-V
modules of the shipped shader programs are embedded into the libraries.
No cmake: a handful of translation units compiled in parallel.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
GEN = os.path.join(BUILD, "gen")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

ICD_LIB = os.path.join(BUILD, "libcpvulkan_gb300.so")
HARNESS_LIB = os.path.join(BUILD, "libcpv_harness.so")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-I" + os.path.join(ROOT, "include"),
            "-I" + os.path.join(CUDA, "include")]

PROGRAMS = ["cube", "texlit", "flatquad", "meshpc", "discard", "nopersp", "points", "fetch", "mrt", "mrti", "storage",
            "separate", "mathx", "calls", "ssbo"]  # index = cpv_program


def _write_if_changed(path, text):
    if os.path.exists(path):
        with open(path) as fh:
            if fh.read() == text:
                return
    with open(path, "w") as fh:
        fh.write(text)


# Kernel headers NVRTC compiles pipeline modules from, in this order (the
# pipeline key hashes them in the same order).
KERNEL_HEADERS = ["cpv_params.h", "cpv_device.cuh", "cpv_raster.cuh", "cpv_stage.cuh", "cpv_pipeline.cuh", "cpv_batch.cuh"]


def _embed_sources():
    kdir = os.path.join(HERE, "csrc", "kernels")
    out = ['#include "../../csrc/runtime/runtime.h"', "namespace cpv::rt {"]
    names, sources = [], []
    for name in KERNEL_HEADERS:
        with open(os.path.join(kdir, name)) as fh:
            src = fh.read()
        if ")CPVSRC" in src:
            raise RuntimeError("delimiter clash in " + name)
        names.append('"%s"' % name)
        sources.append('R"CPVSRC(%s)CPVSRC"' % src)
    out.append("extern const int kKernelHeaderCount = %d;" % len(names))
    out.append("extern const char* const kKernelHeaderNames[] = {%s};" % ", ".join(names))
    out.append("extern const char* const kKernelHeaderSources[] = {\n%s};" % ",\n".join(sources))
    out.append("}")
    _write_if_changed(os.path.join(GEN, "embedded_sources.cpp"), "\n".join(out) + "\n")


def _embed_spirv():
    sdir = os.path.join(HERE, "shaders")
    missing = [p for p in PROGRAMS for s in ("vert", "frag") if not os.path.exists(os.path.join(sdir, "%s.%s.spv" % (p, s)))]
    if missing:
        subprocess.check_call([sys.executable, os.path.join(sdir, "gen_spirv.py"), sdir])
    lines = ["#include <cstddef>", "#include <cstdint>"]
    table = []
    for i, p in enumerate(PROGRAMS):
        for j, s in enumerate(("vert", "frag")):
            with open(os.path.join(sdir, "%s.%s.spv" % (p, s)), "rb") as fh:
                data = fh.read()
            words = [int.from_bytes(data[k:k + 4], "little") for k in range(0, len(data), 4)]
            lines.append("static const uint32_t k_%s_%s[] = {%s};" % (p, s, ",".join("0x%08xu" % w for w in words)))
            table.append("{%d, %d, k_%s_%s, sizeof(k_%s_%s)}" % (i, j, p, s, p, s))
    lines.append("struct SpirvBlob { uint32_t program, stage; const uint32_t* words; size_t bytes; };")
    lines.append("static const SpirvBlob kBlobs[] = {%s};" % ", ".join(table))
    lines.append('extern "C" const uint32_t* cpvh_spirv(uint32_t program, uint32_t stage, size_t* bytes) {')
    lines.append("  for (const auto& b : kBlobs) if (b.program == program && b.stage == stage) { *bytes = b.bytes; return b.words; }")
    lines.append("  *bytes = 0; return nullptr;\n}")
    _write_if_changed(os.path.join(GEN, "shaders_embed.cpp"), "\n".join(lines) + "\n")


def _needs(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _check_arch():
    """Objects built on another machine architecture are discarded."""
    import platform
    import shutil
    stamp = os.path.join(BUILD, "ARCH")
    arch = platform.machine()
    if os.path.isdir(BUILD):
        old = open(stamp).read().strip() if os.path.exists(stamp) else ""
        if old != arch:
            shutil.rmtree(BUILD)
    os.makedirs(GEN, exist_ok=True)
    with open(stamp, "w") as fh:
        fh.write(arch)


def build(verbose=False):
    """Builds what is out of date. Processes that build at the same time (one
    per rank under torchrun) take turns on a lock file."""
    import fcntl
    with open(os.path.join(HERE, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build(verbose)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build(verbose):
    _check_arch()
    _embed_sources()
    _embed_spirv()
    csrc = os.path.join(HERE, "csrc")
    kernels = [os.path.join(csrc, "kernels", f) for f in KERNEL_HEADERS + ["cpv_bin.cuh"]]
    headers = [os.path.join(csrc, "icd", "icd.h"), os.path.join(csrc, "runtime", "runtime.h"), os.path.join(csrc, "spirv", "spirv.h"),
               os.path.join(ROOT, "include", "cpvulkan_gb300.h"), os.path.join(ROOT, "include", "cpv", "vk_subset.h")]
    jobs = []
    objs_icd = []
    for src in ("icd/icd.cpp", "icd/command.cpp", "icd/pipeline.cpp", "icd/sha3.cpp", "spirv/spirv.cpp"):
        path = os.path.join(csrc, src)
        obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs_icd.append(obj)
        if _needs(obj, [path] + headers + kernels):
            jobs.append(["g++"] + CXXFLAGS + ["-fvisibility=hidden", "-c", path, "-o", obj])
    emb = os.path.join(GEN, "embedded_sources.cpp")
    emb_obj = os.path.join(BUILD, "embedded_sources.o")
    objs_icd.append(emb_obj)
    if _needs(emb_obj, [emb] + headers + kernels):
        jobs.append(["g++"] + CXXFLAGS + ["-fvisibility=hidden", "-c", emb, "-o", emb_obj])
    rt_src = os.path.join(csrc, "runtime", "runtime.cu")
    rt_obj = os.path.join(BUILD, "runtime.o")
    objs_icd.append(rt_obj)
    if _needs(rt_obj, [rt_src] + headers + kernels):
        jobs.append([NVCC, ARCH, "-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-I" + os.path.join(ROOT, "include"),
                     "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-c", rt_src, "-o", rt_obj])
    objs_h = []
    for src in ("harness/harness.cpp", "harness/scenes.cpp"):
        path = os.path.join(csrc, src)
        obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs_h.append(obj)
        if _needs(obj, [path] + headers + [os.path.join(ROOT, "include", "cpv_harness.h"), os.path.join(ROOT, "include", "cpv", "scene.h")]):
            jobs.append(["g++"] + CXXFLAGS + ["-c", path, "-o", obj])
    sh = os.path.join(GEN, "shaders_embed.cpp")
    sh_obj = os.path.join(BUILD, "shaders_embed.o")
    objs_h.append(sh_obj)
    if _needs(sh_obj, [sh]):
        jobs.append(["g++"] + CXXFLAGS + ["-c", sh, "-o", sh_obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    libdir = os.path.join(CUDA, "lib64")
    if _needs(ICD_LIB, objs_icd):
        _run(["g++", "-shared", "-o", ICD_LIB] + objs_icd +
             ["-L" + libdir, "-Wl,-rpath," + libdir, "-lcudart_static", "-lnvrtc", "-ldl", "-lpthread", "-lrt"])
    if _needs(HARNESS_LIB, objs_h):
        _run(["g++", "-shared", "-o", HARNESS_LIB] + objs_h + ["-ldl"])
    _write_manifest()
    return ICD_LIB, HARNESS_LIB


def _write_manifest():
    """ICD manifest for a Vulkan loader (the reference's CPVulkan/CPVulkan.json layout)."""
    text = ('{\n  "file_format_version": "1.0.0",\n  "ICD": {\n    "library_path": "%s",\n    "api_version": "1.1.121"\n  }\n}\n' % ICD_LIB)
    _write_if_changed(os.path.join(BUILD, "CPVulkan.json"), text)


if __name__ == "__main__":
    build(verbose=True)
    print(ICD_LIB)
    print(HARNESS_LIB)
