"""Builds oracle/_ref/librefpin.so from the reference's own source files.

TEST INFRASTRUCTURE ONLY: the library is the reference's code for the parts
of the draw path that are plain C++ (no LLVM JIT), used to pin the oracle.

Usage: python extract.py <reference root> <output dir> <c++ compiler>

The functions named in FUNCTIONS are read from the reference files where
they lie, each located by its signature and taken whole (to its closing
brace), written to <output dir>/refpin_src.inc, compiled together with
refpin.cpp (this directory) against shim.h, and the extracted text is
deleted again: only the shared library stays in the output directory, and
nothing extracted is kept in the repository.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# (file relative to the reference root, regex of the definition's first line)
FUNCTIONS = [
    # CPVulkan/CommandBuffer.Draw.cpp
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^enum class InterpolationType$"),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^struct VariableInOutData$"),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^static float EdgeFunction\(const glm::vec2& a, const glm::vec2& b, const glm::vec2& c\)$"),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^static float EdgeFunction\(const glm::vec4& a, const glm::vec4& b, const glm::vec2& c\)$"),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^T SetDatum\(const float points\[size\], const T values\[size\], const float weights\[size\]\)$"),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^void SetDatum\(const VariableInOutData& input, "),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^static bool GetFragmentInput\("),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^static T ApplyBlendFactor\("),
    ("CPVulkan/CommandBuffer.Draw.cpp", r"^static T ApplyBlend\("),
    # CPVulkan/ImageSampler.cpp
    ("CPVulkan/ImageSampler.cpp", r"^static int32_t wrap\(int32_t v, int32_t size, VkSamplerAddressMode addressMode\)$"),
    ("CPVulkan/ImageSampler.cpp", r"^T frac\(T value\)$"),
    ("CPVulkan/ImageSampler.cpp", r"^static T lerp\(T min, T max, double delta\)$"),
    ("CPVulkan/ImageSampler.cpp", r"^ResultType GetPixelLinear\("),
    ("CPVulkan/ImageSampler.cpp", r"^ResultType GetPixelMinMax\("),
    ("CPVulkan/ImageSampler.cpp", r"^ResultType SampleImageOfLevel\("),
    ("CPVulkan/ImageSampler.cpp", r"^ResultType SampleImage\(DeviceState\* deviceState, VkFormat format, gsl::span<uint8_t> data\[MAX_MIP_LEVELS\], "
                                  r"RangeType range\[MAX_MIP_LEVELS\], uint32_t baseLevel, uint32_t levels, CoordinateType coordinates,$"),
]


def take(lines, pattern, path):
    rx = re.compile(pattern)
    hits = [i for i, l in enumerate(lines) if rx.search(l.rstrip("\r\n"))]
    if len(hits) != 1:
        raise SystemExit("%s: %d matches for %r" % (path, len(hits), pattern))
    start = hits[0]
    if start > 0 and lines[start - 1].lstrip().startswith("template<"):
        start -= 1
    depth, seen, end = 0, False, None
    for i in range(hits[0], len(lines)):
        for ch in lines[i]:
            if ch == "{":
                depth += 1
                seen = True
            elif ch == "}":
                depth -= 1
        if seen and depth == 0:
            end = i
            break
    if end is None:
        raise SystemExit("%s: unterminated definition for %r" % (path, pattern))
    return start, end


def main(ref_root, out_dir, cxx):
    os.makedirs(out_dir, exist_ok=True)
    chunks = []
    cache = {}
    for rel, pattern in FUNCTIONS:
        path = os.path.join(ref_root, rel)
        if path not in cache:
            with open(path, encoding="utf-8", errors="replace") as fh:
                cache[path] = fh.readlines()
        lines = cache[path]
        s, e = take(lines, pattern, path)
        chunks.append('#line %d "%s"\n' % (s + 1, path) + "".join(lines[s:e + 1]))
    inc = os.path.join(out_dir, "refpin_src.inc")
    # Blend-op names of extensions the subset header does not carry get
    # distinct placeholder values (the pinned cases never take them).
    text = "\n".join(chunks)
    with open(os.path.join(HERE, "..", "..", "include", "cpv", "vk_subset.h")) as fh:
        known = set(re.findall(r"\b(VK_[A-Z0-9_]+)\b", fh.read()))
    shimmed = set(re.findall(r"\b(VK_[A-Z0-9_]+)\b", open(os.path.join(HERE, "shim.h")).read()))
    missing = sorted(set(re.findall(r"\b(VK_[A-Z0-9_]+)\b", text)) - known - shimmed)
    enums = "".join("#define %s %d\n" % (n, 0x40000000 + i) for i, n in enumerate(missing))
    with open(inc, "w") as fh:
        fh.write(enums + text)
    so = os.path.join(out_dir, "librefpin.so")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I", HERE, "-I", out_dir, "-I",
           os.path.join(HERE, "..", "..", "include"), "-o", so, os.path.join(HERE, "refpin.cpp")]
    try:
        subprocess.check_call(cmd)
    finally:
        os.remove(inc)
    print(so)


if __name__ == "__main__":
    main(*sys.argv[1:4])
