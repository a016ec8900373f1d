"""Pipeline creation on a machine without a GPU (compile-only device):
SPIR-V translation and NVRTC compilation for sm_103a of every shipped shader
program under its fixed-function variants, the pipeline key (SHA3-256 of the
generated source and the kernel headers it includes), and the disk cache."""
import glob
import hashlib
import os

import pytest

import cpvulkan_gb300 as c

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KERNELS = os.path.join(ROOT, "cpvulkan_gb300", "csrc", "kernels")

# (program, variant bits) — bits: 0-1 cull, 2 front CW, 3-4 depth format,
# 5 blend, 6-7 depth op, 8 stencil, 9 BGRA, 10-11 topology, 12 u16 indices,
# 13 depth write off, 14 nearest + mirror/border sampler, 15 LOD bias,
# 16 point/line topologies (10-11 then: points, lines, line strip), 17 wide lines,
# 18 logic op (op in bits 20-23), 19 colour write mask (mask in bits 24-27),
# 28-29 depth bounds, 30 depth-only pass
PROGRAMS = [
    (c.PROGRAM_CUBE, 0x0), (c.PROGRAM_CUBE, 0x18 | 0x100), (c.PROGRAM_CUBE, 0x20 | 0x200 | 0x400),
    (c.PROGRAM_TEXLIT, 0x10 | 0x4000), (c.PROGRAM_FLATQUAD, 0x20), (c.PROGRAM_MESHPC, 0x10 | 0x2 | 0x4),
    (c.PROGRAM_DISCARD, 0x10), (c.PROGRAM_NOPERSP, 0x8 | 0x800),
    (c.PROGRAM_POINTS, 0x10000 | 0x10), (c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000), (c.PROGRAM_NOPERSP, 0x10000 | 0x800 | 0x8),
    (c.PROGRAM_CUBE, 0x40000 | (6 << 20) | 0x10), (c.PROGRAM_FLATQUAD, 0x20 | 0x80000 | (0x5 << 24)),
    (c.PROGRAM_CUBE, 0x18 | 0x100 | (2 << 28)), (c.PROGRAM_TEXLIT, 0x40000000 | 0x10), (c.PROGRAM_FETCH, 0x0),
]


@pytest.fixture
def compile_ctx(native, monkeypatch, tmp_path):
    monkeypatch.setenv("CPV_COMPILE_ONLY", "1")
    monkeypatch.setenv("CPV_DUMP_DIR", str(tmp_path))
    ctx = c.Context()
    yield ctx, tmp_path
    ctx.close()


@pytest.mark.parametrize("program,variant", PROGRAMS)
def test_program_compiles(compile_ctx, program, variant):
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [program, variant, 32, 32, 4]))
    sources = glob.glob(str(dump / "pipeline_*.cu"))
    assert sources
    text = open(sources[0]).read()
    assert "cpv_vs_run" in text and "cpv_fs_run" in text


def test_pipeline_key_is_sha3_of_source_and_kernels(compile_ctx):
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_TEXLIT, 0x10, 32, 32, 4]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    keyed = open(path, "rb").read()
    from cpvulkan_gb300.native_build import KERNEL_HEADERS
    for h in KERNEL_HEADERS:
        keyed += open(os.path.join(KERNELS, h), "rb").read()
    assert os.path.basename(path) == "pipeline_%s.cu" % hashlib.sha3_256(keyed).hexdigest()[:12]


def test_disk_cache_round_trip(native, monkeypatch, tmp_path):
    monkeypatch.setenv("CPV_COMPILE_ONLY", "1")
    monkeypatch.setenv("CPV_CACHE_DIR", str(tmp_path))
    scene = c.Scene(c.PROGRAM, 1, [c.PROGRAM_FLATQUAD, 0x20, 32, 32, 4])
    ctx = c.Context()
    ctx.compile_pipelines(scene)
    ctx.close()
    cubins = glob.glob(str(tmp_path / "*.cubin"))
    assert len(cubins) == 1 and os.path.getsize(cubins[0]) > 1000
    mtime = os.path.getmtime(cubins[0])
    ctx = c.Context()  # a new device: the cubin comes from the disk cache
    ctx.compile_pipelines(scene)
    ctx.close()
    assert os.path.getmtime(cubins[0]) == mtime


@pytest.mark.parametrize("tile", ["8", "32"])
def test_tile_sizes_compile(native, monkeypatch, tile):
    monkeypatch.setenv("CPV_COMPILE_ONLY", "1")
    monkeypatch.setenv("CPV_TILE", tile)
    ctx = c.Context()
    ctx.compile_pipelines(c.Scene(c.HEIGHTFIELD, 1, [16, 64, 64]))
    ctx.close()



def _module_source(compile_ctx, program, variant):
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [program, variant, 32, 32, 4]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    return open(path).read()


@pytest.mark.parametrize("program,variant,expect", [
    # lines need the fourth edge in every coverage test of their module
    (c.PROGRAM_CUBE, 0x10000 | 0x400, {"CPV_ANY_LINES": "1", "CPV_TOPOLOGY": "1"}),
    (c.PROGRAM_POINTS, 0x10000, {"CPV_ANY_LINES": "0", "CPV_TOPOLOGY": "0"}),
    # flat shading: the immediate schedule, 128-primitive batches, a 7-CTA register budget
    (c.PROGRAM_FLATQUAD, 0x20, {"CPV_FS_CONSTANT": "1", "CPV_SCHEDULE": "0", "CPV_BATCH": "128", "CPV_PLAIN_MIN_BLOCKS": "7",
                                "CPV_BLEND_TABLE": "1"}),
    # interpolated colour: sparse schedule, 256-primitive batches, 24 fragments a pixel
    (c.PROGRAM_CUBE, 0x10, {"CPV_SCHEDULE": "2", "CPV_BATCH": "256", "CPV_SLOT_DEPTH": "24", "CPV_RT_MIN_BLOCKS": "5"}),
    # texture sampling: 16 fragments a pixel, a 4-CTA budget for the batched raster
    (c.PROGRAM_TEXLIT, 0x10, {"CPV_SCHEDULE": "2", "CPV_SLOT_DEPTH": "16", "CPV_RT_MIN_BLOCKS": "4"}),
    # a logic op turns blending (and so the blend tables) off
    (c.PROGRAM_FLATQUAD, 0x20 | 0x40000 | (9 << 20), {"CPV_LOGIC": "1", "CPV_LOGIC_OP": "9", "CPV_BLEND": "0", "CPV_BLEND_TABLE": "0"}),
    (c.PROGRAM_CUBE, 0x80000 | (0xA << 24), {"CPV_LOGIC": "0", "CPV_WRITE_MASK": "10u"}),
    # static depth bounds as float bit patterns (0.3f, 1.0f)
    (c.PROGRAM_CUBE, 0x10 | (2 << 28), {"CPV_DEPTH_BOUNDS": "1", "CPV_MIN_DEPTH_BOUNDS": "__uint_as_float(1050253722u)",
                                       "CPV_MAX_DEPTH_BOUNDS": "__uint_as_float(1065353216u)"}),
    # no depth attachment: no test
    (c.PROGRAM_FLATQUAD, 0x20 | (2 << 28), {"CPV_DEPTH_BOUNDS": "0"}),
    # a depth-only pass: no colour format, blending off
    (c.PROGRAM_FLATQUAD, 0x40000000 | 0x8 | 0x20, {"CPV_COLOR_FORMAT": "0", "CPV_DEPTH_FORMAT": "124", "CPV_BLEND": "0"}),
])
def test_module_configuration(compile_ctx, program, variant, expect):
    """The fixed-function and schedule macros a pipeline's module is compiled with."""
    text = _module_source(compile_ctx, program, variant)
    for name, value in expect.items():
        assert "#define %s %s\n" % (name, value) in text, (name, value)


@pytest.mark.parametrize("subpasses,colour", [("2", "37"), ("2:0", "0")])
def test_pipeline_takes_its_subpass_formats(compile_ctx, monkeypatch, subpasses, colour):
    """A pipeline is compiled for the attachments of the subpass it is created
    for: in a render pass whose subpass 0 references only the depth
    attachment and subpass 1 colour and depth, a subpass-1 pipeline writes
    RGBA8 colour and a subpass-0 pipeline none."""
    monkeypatch.setenv("CPVH_SUBPASSES", subpasses)
    text = _module_source(compile_ctx, c.PROGRAM_CUBE, 0x18 | 0x100)
    assert "#define CPV_COLOR_FORMAT %s\n" % colour in text
    assert "#define CPV_DEPTH_FORMAT 130\n" in text


@pytest.mark.parametrize("config,params", [
    (c.BATCH, [24, 2000, 320, 200]),
    (c.PROGRAM, [c.PROGRAM_POINTS, 0x10000 | 0x20, 32, 32, 4]),
    (c.PROGRAM, [c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000, 32, 32, 4]),
    (c.PROGRAM, [c.PROGRAM_TEXLIT, 0x10, 32, 32, 4]),
])
def test_batched_module_compiles(native, monkeypatch, tmp_path, config, params):
    """Recording a render pass that runs batched compiles its batched module
    (every pipeline of the pass in one NVRTC module) at vkEndCommandBuffer;
    on the compile-only device that must succeed for triangle, point and
    line pipelines. Each compiled module leaves a cubin in the disk cache."""
    dump, cache = tmp_path / "dump", tmp_path / "cache"
    dump.mkdir()
    cache.mkdir()
    monkeypatch.setenv("CPV_COMPILE_ONLY", "1")
    monkeypatch.setenv("CPV_DUMP_DIR", str(dump))
    monkeypatch.setenv("CPV_CACHE_DIR", str(cache))
    monkeypatch.setenv("CPVH_RECORD_ONLY", "1")
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    monkeypatch.setenv("CPV_AUTOTUNE", "0")
    ctx = c.Context()
    try:
        r = c.Renderer(ctx, c.Scene(config, 1, params))
        r.close()
    finally:
        ctx.close()
    batch = glob.glob(str(dump / "batch_*.cu"))
    assert batch, "no batched module was composed"
    assert "#include \"cpv_batch.cuh\"" in open(batch[0]).read()
    sources = glob.glob(str(dump / "*.cu"))
    assert len(glob.glob(str(cache / "*.cubin"))) >= len(sources), c.icd_last_error()


@pytest.mark.parametrize("fmt,expect", [(38, "cpv_decode_norm"), (92, "cpv_decode_norm"), (44, "cpv_decode_norm"), (97, "cpv_half_to_float")])
def test_vertex_attribute_formats_translate(compile_ctx, fmt, expect):
    """Normalised 8/16-bit and half-float colour attributes compile to the
    decoder the reference's vertex fetch uses for them."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, 0x10, 32, 32, 4, fmt]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    assert expect in open(path).read()


@pytest.mark.parametrize("fmt", [76, 83])
def test_half_attribute_of_other_width_rejected(compile_ctx, fmt):
    """A half-float attribute narrower than its vec4 input is rejected at
    pipeline creation (the reference aborts on the width mismatch)."""
    ctx, _ = compile_ctx
    with pytest.raises(RuntimeError, match="half-float vertex attribute"):
        ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, 0x10, 32, 32, 4, fmt]))


@pytest.mark.parametrize("k,scale", [(0, "int32_t(3)"), (5, "int32_t(5)")])
def test_fetch_program_translation(compile_ctx, k, scale):
    """OpImage / OpImageFetch become a level-0 fetch, OpBitCount a population
    count, OpCopyMemory a copy of the variable, and the specialisation
    constant (overridden by VkSpecializationInfo when given) feeds the
    folded OpSpecConstantOp expression."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_FETCH, 0x0, 32, 32, 4, k]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    text = open(path).read()
    assert "cpv_fetch(P.tex[" in text and "__popc(" in text
    assert scale in text and "(uint32_t)(int32_t(8))" in text


def test_secondary_command_buffers_record_batched_pass(native, monkeypatch, tmp_path):
    """Draws recorded in secondary command buffers and run by
    vkCmdExecuteCommands become the primary's own commands: a pass of many
    draws composed that way is compiled as one batched module when the
    primary is ended."""
    dump = tmp_path / "dump"
    dump.mkdir()
    for k, v in {"CPV_COMPILE_ONLY": "1", "CPV_DUMP_DIR": str(dump), "CPVH_RECORD_ONLY": "1", "CPVH_SECONDARY": "1",
                 "CPV_AUTOTUNE": "0"}.items():
        monkeypatch.setenv(k, v)
    ctx = c.Context()
    try:
        c.Renderer(ctx, c.Scene(c.BATCH, 1, [24, 2000, 320, 200])).close()
    finally:
        ctx.close()
    assert glob.glob(str(dump / "batch_*.cu"))


COLOUR_ATTACHMENTS = [(9, 1, 1, 8, 0), (16, 2, 2, 8, 0), (38, 4, 4, 8, 1), (70, 2, 1, 16, 0), (77, 4, 2, 16, 0), (83, 4, 2, 16, 2),
                      (100, 4, 1, 32, 2), (91, 8, 4, 16, 0), (97, 8, 4, 16, 2), (103, 8, 2, 32, 2), (109, 16, 4, 32, 2)]


@pytest.mark.parametrize("fmt,nbytes,channels,bits,kind", COLOUR_ATTACHMENTS)
@pytest.mark.parametrize("variant", [0x10, 0x20 | 0x80000 | (0x5 << 24)])
def test_colour_attachment_formats_compile(compile_ctx, fmt, nbytes, channels, bits, kind, variant):
    """A colour attachment in any of the draw path's formats compiles with
    the format's layout: texel bytes, channels, bits per channel and kind
    (0 UNORM, 1 SNORM, 2 SFLOAT); blending never takes the RGBA8 tables."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_FLATQUAD, variant, 32, 32, 4, 0, fmt]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    text = open(path).read()
    for name, value in (("BYTES", nbytes), ("CHANNELS", channels), ("BITS", bits), ("KIND", kind)):
        assert "#define CPV_CF_%s %d\n" % (name, value) in text
    assert "#define CPV_BLEND_TABLE 0\n" in text


@pytest.mark.parametrize("fmt", [70, 77, 83, 100, 91, 109])
def test_logic_op_on_wide_colour_format_rejected(compile_ctx, fmt):
    """A logic op is accepted on 8-bit normalised colour attachments only."""
    ctx, _ = compile_ctx
    with pytest.raises(RuntimeError, match="logic op on colour format"):
        ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, 0x40000 | (6 << 20), 32, 32, 4, 0, fmt]))


def test_logic_op_on_8bit_colour_formats_compiles(compile_ctx):
    ctx, dump = compile_ctx
    for fmt in (9, 16, 38):
        ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, 0x40000 | (6 << 20), 32, 32, 4, 0, fmt]))
    assert len(glob.glob(str(dump / "pipeline_*.cu"))) == 3


def test_colour_attachments_compile_and_reject(native, monkeypatch, tmp_path):
    """A subpass of eight colour references (one unused) compiles per draw
    and batched; a fragment shader without an output for a used attachment
    is rejected at pipeline creation (the reference looks the location up
    with std::map::at)."""
    for k, v in {"CPV_COMPILE_ONLY": "1", "CPV_CACHE_DIR": str(tmp_path), "CPVH_RECORD_ONLY": "1", "CPV_AUTOTUNE": "0",
                 "CPV_BATCH_MIN_DRAWS": "1"}.items():
        monkeypatch.setenv(k, v)
    fmts = 44 | (83 << 8) | (100 << 16) | (9 << 24) | (38 << 32) | (0 << 40) | (77 << 48)
    ctx = c.Context()
    try:
        c.Renderer(ctx, c.Scene(c.PROGRAM, 1, [c.PROGRAM_MRT, 0x10, 32, 32, 4, 0, 0, fmts, 0x0201])).close()
        assert "batched module compiled" in c.icd_last_error()
        # integer outputs into integer formats of every width
        ints = 41 | (42 << 8) | (98 << 16)
        c.Renderer(ctx, c.Scene(c.PROGRAM, 1, [c.PROGRAM_MRTI, 0x10, 32, 32, 4, 0, 99, ints, 0x01])).close()
        assert "batched module compiled" in c.icd_last_error()
        with pytest.raises(RuntimeError):
            c.Renderer(ctx, c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, 0x10, 32, 32, 4, 0, 0, 37, 0]))
        assert "no output for colour attachment 1" in c.icd_last_error()
        # 8- and 16-byte texels: the first attachment only
        c.Renderer(ctx, c.Scene(c.PROGRAM, 1, [c.PROGRAM_MRTI, 0x10, 32, 32, 4, 0, 107, 98, 0])).close()
        assert "batched module compiled" in c.icd_last_error()
        with pytest.raises(RuntimeError):
            c.Renderer(ctx, c.Scene(c.PROGRAM, 1, [c.PROGRAM_MRTI, 0x10, 32, 32, 4, 0, 98, 107, 0]))
        assert "an 8- or 16-byte colour format after the first attachment" in c.icd_last_error()
    finally:
        ctx.close()


def test_spec_lod_module(compile_ctx, monkeypatch):
    """CPV_SPEC_LOD=1 compiles a fragment shader's implicit-LOD sampling as
    quad-derivative sites (cpv_sample_quad, CPV_LOD_SITES); without it the
    module samples at the reference's λ 0 and has no site."""
    ctx, dump = compile_ctx
    scene = [c.PROGRAM_TEXLIT, 0x10, 32, 32, 4]
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, scene))
    (plain,) = glob.glob(str(dump / "pipeline_*.cu"))
    monkeypatch.setenv("CPV_SPEC_LOD", "1")
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, scene))
    (spec,) = set(glob.glob(str(dump / "pipeline_*.cu"))) - {plain}
    plain, spec = open(plain).read(), open(spec).read()
    assert "#define CPV_LOD_SITES 0\n" in plain and "cpv_sample_quad(" not in plain
    assert "#define CPV_LOD_SITES 1\n" in spec and "cpv_sample_quad(P.tex[0]" in spec and "cpv_lod, 0)" in spec


def test_image_binding_modules(compile_ctx):
    """A storage image read by imageLoad compiles to a level-0 texel fetch
    (cpv_fetch) and a sampled image joined with a sampler from another
    binding to an ordinary texture sample, each in texture slot 0."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_STORAGE, 0x10, 32, 32, 4]))
    (storage,) = glob.glob(str(dump / "pipeline_*.cu"))
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_SEPARATE, 0x10, 32, 32, 4]))
    (separate,) = set(glob.glob(str(dump / "pipeline_*.cu"))) - {storage}
    storage, separate = open(storage).read(), open(separate).read()
    assert "cpv_fetch(P.tex[0]" in storage and "cpv_sample(" not in storage
    assert "cpv_sample(P.tex[0]" in separate


def test_glsl_builtins_translate(compile_ctx):
    """NMin, NMax, NClamp, FindSMsb, FindILsb, FindUMsb, SSign and Reflect
    (GLSL.std.450 71-81, 7) translate to the device helpers that restate
    the reference's definitions."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_MATHX, 0x10, 32, 32, 4]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    text = open(path).read()
    for fn in ("cpv_glsl_nclamp(", "cpv_glsl_nmin(", "cpv_glsl_nmax(", "cpv_find_smsb(", "cpv_find_ilsb(", "cpv_find_umsb(", "cpv_glsl_reflect("):
        assert fn in text, fn


def test_function_calls_translate(compile_ctx):
    """Functions other than the entry point become lambdas of the stage
    function, callees first; a pointer parameter is a reference to the
    caller's variable, and a discard inside one ends the invocation."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_CALLS, 0x10, 32, 32, 4]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    text = open(path).read()
    assert text.count("= [&](") == 2
    assert "cvec<float, 4>& v" in text and "cpv_killed = true;" in text and "if (cpv_killed) return true;" in text


def test_storage_buffer_reads_translate(compile_ctx):
    """A read-only storage buffer (BufferBlock, runtime array) is read with
    the uniform buffers' bounds-checked explicit-layout loads, from its own
    buffer slot."""
    ctx, dump = compile_ctx
    ctx.compile_pipelines(c.Scene(c.PROGRAM, 1, [c.PROGRAM_SSBO, 0x10, 32, 32, 4]))
    (path,) = glob.glob(str(dump / "pipeline_*.cu"))
    text = open(path).read()
    assert "P.ubo[1], P.ubo_bytes[1]" in text

