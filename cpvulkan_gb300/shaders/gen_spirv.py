#!/usr/bin/env python3
"""Emit the SPIR-V modules of the shader programs the harness renders with.

There is no GLSL compiler in this image, so the vertex/fragment modules are
assembled directly from the SPIR-V 1.0 binary specification (word layout,
opcode and enumerant numbers). Each program mirrors a GLSL shader given in its
docstring; the instruction sequence is what the CPU oracle restates op for op.

Usage: python gen_spirv.py [outdir]   (default: this directory)
Writes <program>.vert.spv / <program>.frag.spv.
"""
import os
import struct
import sys

# --- opcodes (SPIR-V 1.0) ---------------------------------------------------
OP = dict(
    Name=5, MemberName=6, ExtInstImport=11, ExtInst=12, MemoryModel=14, EntryPoint=15, ExecutionMode=16,
    Capability=17, TypeVoid=19, TypeBool=20, TypeInt=21, TypeFloat=22, TypeVector=23, TypeMatrix=24,
    TypeImage=25, TypeSampledImage=27, TypeArray=28, TypeStruct=30, TypePointer=32, TypeFunction=33,
    Constant=43, ConstantComposite=44, Function=54, FunctionEnd=56, Variable=59, Load=61, Store=62,
    AccessChain=65, Decorate=71, MemberDecorate=72, VectorShuffle=79, CompositeConstruct=80,
    CompositeExtract=81, ImageSampleImplicitLod=87, FAdd=129, FSub=131, FMul=133, FDiv=136,
    VectorTimesScalar=142, MatrixTimesVector=145, Dot=148, FOrdGreaterThan=186, SelectionMerge=247,
    Label=248, Branch=249, BranchConditional=250, Kill=252, Return=253, SpecConstant=50, SpecConstantOp=52,
    CopyMemory=63, ImageFetch=95, Image=100, ConvertFToS=110, ConvertSToF=111, IAdd=128, IMul=132, BitwiseXor=198,
    BitCount=205, ConvertFToU=109, Bitcast=124, TypeSampler=26, SampledImage=86, ImageRead=98, ISub=130,
    FunctionParameter=55, FunctionCall=57, ReturnValue=254, TypeRuntimeArray=29,
)
DEC = dict(SpecId=1, Block=2, ColMajor=5, MatrixStride=7, BuiltIn=11, NoPerspective=13, Flat=14, Location=30, Binding=33,
           DescriptorSet=34, Offset=35, BufferBlock=3, ArrayStride=6, NonWritable=24)
SC = dict(UniformConstant=0, Input=1, Uniform=2, Output=3, Function=7, PushConstant=9)
BUILTIN = dict(Position=0, PointSize=1, ClipDistance=3, CullDistance=4)
GLSL = dict(FMax=40, Normalize=69, SSign=7, Reflect=71, FindILsb=73, FindSMsb=74, FindUMsb=75, NMin=79, NMax=80, NClamp=81)


def _str_words(s):
    b = s.encode() + b"\0"
    b += b"\0" * ((4 - len(b) % 4) % 4)
    return list(struct.unpack("<%dI" % (len(b) // 4), b))


def _f32(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


class Module:
    """Minimal SPIR-V module builder with type/constant de-duplication."""

    def __init__(self, model):
        self.model = model  # 0 vertex, 4 fragment
        self.next_id = 1
        self.caps, self.ext, self.mem, self.entry, self.modes = [], [], [], [], []
        self.names, self.annot, self.types, self.body = [], [], [], []
        self.cache = {}
        self.interface = []
        self.glsl = self.id()
        self.ext.append(self._ins("ExtInstImport", [self.glsl] + _str_words("GLSL.std.450")))

    def id(self):
        i = self.next_id
        self.next_id += 1
        return i

    @staticmethod
    def _ins(op, words):
        return [((len(words) + 1) << 16) | OP[op]] + list(words)

    def _type(self, key, op, words_fn):
        if key not in self.cache:
            i = self.id()
            self.types.append(self._ins(op, [i] + words_fn()))
            self.cache[key] = i
        return self.cache[key]

    def _const(self, key, op, type_fn, words_fn):
        """Constants put the result type before the result id."""
        if key not in self.cache:
            t = type_fn()
            words = words_fn()
            i = self.id()
            self.types.append(self._ins(op, [t, i] + words))
            self.cache[key] = i
        return self.cache[key]

    # types
    def void(self): return self._type(("void",), "TypeVoid", lambda: [])
    def bool(self): return self._type(("bool",), "TypeBool", lambda: [])
    def int(self): return self._type(("int",), "TypeInt", lambda: [32, 1])
    def float(self): return self._type(("float",), "TypeFloat", lambda: [32])
    def vec(self, n): return self._type(("vec", n), "TypeVector", lambda: [self.float(), n])
    def mat4(self): return self._type(("mat4",), "TypeMatrix", lambda: [self.vec(4), 4])
    def ptr(self, sc, t): return self._type(("ptr", sc, t), "TypePointer", lambda: [SC[sc], t])
    def fn_void(self): return self._type(("fnvoid",), "TypeFunction", lambda: [self.void()])

    def array(self, t, n):
        return self._type(("arr", t, n), "TypeArray", lambda: [t, self.const_int(n)])

    def struct(self, key, members):
        return self._type(("struct", key), "TypeStruct", lambda: list(members))

    def ivec(self, n): return self._type(("ivec", n), "TypeVector", lambda: [self.int(), n])
    def uint(self): return self._type(("uint",), "TypeInt", lambda: [32, 0])
    def uvec(self, n): return self._type(("uvec", n), "TypeVector", lambda: [self.uint(), n])

    def image_2d(self):
        return self._type(("img2d",), "TypeImage", lambda: [self.float(), 1, 0, 0, 0, 1, 0])

    def sampled_image_2d(self):
        img = self.image_2d()
        return self._type(("simg2d",), "TypeSampledImage", lambda: [img])

    def storage_image_2d_rgba8(self):
        # Sampled 2 (storage), ImageFormat Rgba8 (4)
        return self._type(("stimg2d",), "TypeImage", lambda: [self.float(), 1, 0, 0, 0, 2, 4])

    def sampler(self):
        return self._type(("sampler",), "TypeSampler", lambda: [])

    def spec_const_int(self, default, spec_id):
        c = self._const(("sci", spec_id), "SpecConstant", self.int, lambda: [default & 0xFFFFFFFF])
        self.decorate(c, "SpecId", spec_id)
        return c

    def spec_op(self, t, opname, *operands):
        return self._const(("sop", t, opname) + tuple(operands), "SpecConstantOp", lambda: t, lambda: [OP[opname]] + list(operands))

    def local(self, t):
        """A Function-storage variable: call first in the entry block."""
        return self.op("Variable", self.ptr("Function", t), SC["Function"])

    # constants
    def const_f(self, x):
        return self._const(("cf", _f32(x)), "Constant", self.float, lambda: [_f32(x)])

    def const_int(self, x):
        return self._const(("ci", x), "Constant", self.int, lambda: [x & 0xFFFFFFFF])

    # declarations
    def decorate(self, target, dec, *lits):
        self.annot.append(self._ins("Decorate", [target, DEC[dec]] + list(lits)))

    def member_decorate(self, st, member, dec, *lits):
        self.annot.append(self._ins("MemberDecorate", [st, member, DEC[dec]] + list(lits)))

    def name(self, target, s):
        self.names.append(self._ins("Name", [target] + _str_words(s)))

    def variable(self, sc, t, name=None):
        v = self.id()
        self.types.append(self._ins("Variable", [self.ptr(sc, t), v, SC[sc]]))
        if name:
            self.name(v, name)
        if sc in ("Input", "Output"):
            self.interface.append(v)
        return v

    # instructions in the function body
    def op(self, opname, rtype, *args):
        r = self.id()
        self.body.append(self._ins(opname, [rtype, r] + list(args)))
        return r

    def op_void(self, opname, *args):
        self.body.append(self._ins(opname, list(args)))

    def load(self, t, p): return self.op("Load", t, p)
    def store(self, p, v): self.op_void("Store", p, v)
    def access(self, sc, t, base, *idx): return self.op("AccessChain", self.ptr(sc, t), base, *idx)
    def ext_inst(self, t, inst, *args): return self.op("ExtInst", t, self.glsl, GLSL[inst], *args)
    def label(self):
        lbl = self.id()
        self.body.append(self._ins("Label", [lbl]))
        return lbl

    def per_vertex_block(self):
        """gl_PerVertex { vec4 Position; float PointSize; float ClipDistance[1]; float CullDistance[1]; }"""
        f = self.float()
        arr = self.array(f, 1)
        st = self.struct("gl_PerVertex", [self.vec(4), f, arr, arr])
        self.member_decorate(st, 0, "BuiltIn", BUILTIN["Position"])
        self.member_decorate(st, 1, "BuiltIn", BUILTIN["PointSize"])
        self.member_decorate(st, 2, "BuiltIn", BUILTIN["ClipDistance"])
        self.member_decorate(st, 3, "BuiltIn", BUILTIN["CullDistance"])
        self.decorate(st, "Block")
        return st, self.variable("Output", st, "gl_PerVertex")

    def ubo_block(self, key, members, offsets, binding, set_=0, sc="Uniform"):
        st = self.struct(key, members)
        for i, off in enumerate(offsets):
            self.member_decorate(st, i, "Offset", off)
            if members[i] == self.mat4():
                self.member_decorate(st, i, "ColMajor")
                self.member_decorate(st, i, "MatrixStride", 16)
        self.decorate(st, "Block")
        v = self.variable(sc, st, key.lower())
        if sc == "Uniform":
            self.decorate(v, "DescriptorSet", set_)
            self.decorate(v, "Binding", binding)
        return v

    def assemble(self, body_fn):
        """body_fn(mod) emits the entry function body after its first label."""
        fn = self.id()
        self.body.append(self._ins("Function", [self.void(), fn, 0, self.fn_void()]))
        self.label()
        body_fn(self)
        self.body.append(self._ins("FunctionEnd", []))
        self.caps.append(self._ins("Capability", [1]))
        self.mem.append(self._ins("MemoryModel", [0, 1]))
        self.entry.append(self._ins("EntryPoint", [self.model, fn] + _str_words("main") + self.interface))
        if self.model == 4:
            self.modes.append(self._ins("ExecutionMode", [fn, 7]))  # OriginUpperLeft
        words = [0x07230203, 0x00010000, 0, self.next_id, 0]
        for sec in (self.caps, self.ext, self.mem, self.entry, self.modes, self.names, self.annot, self.types,
                    self.body):
            for ins in sec:
                words += ins
        return struct.pack("<%dI" % len(words), *words)


# --- programs -----------------------------------------------------------------

def cube_vert():
    """layout(set=0,binding=0) uniform UBO { mat4 mvp; };
    layout(location=0) in vec4 pos; layout(location=1) in vec4 inColor;
    layout(location=0) out vec4 outColor;
    void main() { outColor = inColor; gl_Position = mvp * pos; }"""
    m = Module(0)
    v4, mat = m.vec(4), m.mat4()
    ubo = m.ubo_block("UBO", [mat], [0], binding=0)
    pos = m.variable("Input", v4, "pos")
    m.decorate(pos, "Location", 0)
    col = m.variable("Input", v4, "inColor")
    m.decorate(col, "Location", 1)
    out = m.variable("Output", v4, "outColor")
    m.decorate(out, "Location", 0)
    pv_t, pv = m.per_vertex_block()

    def body(m):
        c = m.load(v4, col)
        m.store(out, c)
        mp = m.access("Uniform", mat, ubo, m.const_int(0))
        mv = m.load(mat, mp)
        p = m.load(v4, pos)
        r = m.op("MatrixTimesVector", v4, mv, p)
        dst = m.access("Output", v4, pv, m.const_int(0))
        m.store(dst, r)
        m.op_void("Return")
    return m.assemble(body)


def points_vert():
    """cube_vert plus gl_PointSize = inColor.a * 16.0 (the gl_PerVertex member)."""
    m = Module(0)
    v4, mat, f = m.vec(4), m.mat4(), m.float()
    ubo = m.ubo_block("UBO", [mat], [0], binding=0)
    pos = m.variable("Input", v4, "pos")
    m.decorate(pos, "Location", 0)
    col = m.variable("Input", v4, "inColor")
    m.decorate(col, "Location", 1)
    out = m.variable("Output", v4, "outColor")
    m.decorate(out, "Location", 0)
    pv_t, pv = m.per_vertex_block()

    def body(m):
        c = m.load(v4, col)
        m.store(out, c)
        mp = m.access("Uniform", mat, ubo, m.const_int(0))
        mv = m.load(mat, mp)
        p = m.load(v4, pos)
        r = m.op("MatrixTimesVector", v4, mv, p)
        m.store(m.access("Output", v4, pv, m.const_int(0)), r)
        a = m.op("CompositeExtract", f, c, 3)
        size = m.op("FMul", f, a, m.const_f(16.0))
        m.store(m.access("Output", f, pv, m.const_int(1)), size)
        m.op_void("Return")
    return m.assemble(body)


def colour_frag(decoration=None, discard=False):
    """layout(location=0) [flat|noperspective] in vec4 color; layout(location=0) out vec4 o;
    void main() { [if (color.r > 0.5) discard;] o = color; }"""
    m = Module(4)
    v4, f = m.vec(4), m.float()
    col = m.variable("Input", v4, "color")
    m.decorate(col, "Location", 0)
    if decoration:
        m.decorate(col, decoration)
    out = m.variable("Output", v4, "o")
    m.decorate(out, "Location", 0)

    def body(m):
        c = m.load(v4, col)
        if discard:
            r = m.op("CompositeExtract", f, c, 0)
            cond = m.op("FOrdGreaterThan", m.bool(), r, m.const_f(0.5))
            kill_lbl, merge_lbl = m.id(), m.id()
            m.op_void("SelectionMerge", merge_lbl, 0)
            m.op_void("BranchConditional", cond, kill_lbl, merge_lbl)
            m.body.append(m._ins("Label", [kill_lbl]))
            m.op_void("Kill")
            m.body.append(m._ins("Label", [merge_lbl]))
        m.store(out, c)
        m.op_void("Return")
    return m.assemble(body)


def texlit_vert():
    """layout(set=0,binding=0) uniform UBO { mat4 mvp; vec4 light; };
    layout(location=0) in vec3 pos; layout(location=1) in vec2 uv; layout(location=2) in vec3 normal;
    layout(location=0) out vec2 vUV; layout(location=1) out vec3 vN;
    void main() { vUV = uv; vN = normal; gl_Position = mvp * vec4(pos, 1.0); }"""
    m = Module(0)
    v2, v3, v4, mat, f = m.vec(2), m.vec(3), m.vec(4), m.mat4(), m.float()
    ubo = m.ubo_block("UBO", [mat, v4], [0, 64], binding=0)
    pos = m.variable("Input", v3, "pos"); m.decorate(pos, "Location", 0)
    uv = m.variable("Input", v2, "uv"); m.decorate(uv, "Location", 1)
    nrm = m.variable("Input", v3, "normal"); m.decorate(nrm, "Location", 2)
    ouv = m.variable("Output", v2, "vUV"); m.decorate(ouv, "Location", 0)
    on = m.variable("Output", v3, "vN"); m.decorate(on, "Location", 1)
    pv_t, pv = m.per_vertex_block()

    def body(m):
        m.store(ouv, m.load(v2, uv))
        m.store(on, m.load(v3, nrm))
        mv = m.load(mat, m.access("Uniform", mat, ubo, m.const_int(0)))
        p = m.load(v3, pos)
        p4 = m.op("CompositeConstruct", v4, p, m.const_f(1.0))
        r = m.op("MatrixTimesVector", v4, mv, p4)
        m.store(m.access("Output", v4, pv, m.const_int(0)), r)
        m.op_void("Return")
    return m.assemble(body)


def texlit_frag():
    """layout(set=0,binding=0) uniform UBO { mat4 mvp; vec4 light; };
    layout(set=0,binding=1) uniform sampler2D tex;
    layout(location=0) in vec2 uv; layout(location=1) in vec3 n; layout(location=0) out vec4 o;
    void main() { vec4 c = texture(tex, uv); float l = max(dot(normalize(n), light.xyz), 0.0);
                  o = vec4(c.xyz * l, c.w); }"""
    m = Module(4)
    v2, v3, v4, mat, f = m.vec(2), m.vec(3), m.vec(4), m.mat4(), m.float()
    ubo = m.ubo_block("UBO", [mat, v4], [0, 64], binding=0)
    simg = m.sampled_image_2d()
    tex = m.variable("UniformConstant", simg, "tex")
    m.decorate(tex, "DescriptorSet", 0)
    m.decorate(tex, "Binding", 1)
    uv = m.variable("Input", v2, "uv"); m.decorate(uv, "Location", 0)
    n = m.variable("Input", v3, "n"); m.decorate(n, "Location", 1)
    out = m.variable("Output", v4, "o"); m.decorate(out, "Location", 0)

    def body(m):
        s = m.load(simg, tex)
        c = m.op("ImageSampleImplicitLod", v4, s, m.load(v2, uv))
        nn = m.ext_inst(v3, "Normalize", m.load(v3, n))
        light = m.load(v4, m.access("Uniform", v4, ubo, m.const_int(1)))
        lxyz = m.op("VectorShuffle", v3, light, light, 0, 1, 2)
        d = m.op("Dot", f, nn, lxyz)
        l = m.ext_inst(f, "FMax", d, m.const_f(0.0))
        cxyz = m.op("VectorShuffle", v3, c, c, 0, 1, 2)
        rgb = m.op("VectorTimesScalar", v3, cxyz, l)
        cw = m.op("CompositeExtract", f, c, 3)
        m.store(out, m.op("CompositeConstruct", v4, rgb, cw))
        m.op_void("Return")
    return m.assemble(body)


def flatquad_vert():
    """layout(location=0) in vec2 pos; layout(location=1) in vec4 color; layout(location=0) out vec4 vColor;
    void main() { vColor = color; gl_Position = vec4(pos, 0.0, 1.0); }"""
    m = Module(0)
    v2, v4 = m.vec(2), m.vec(4)
    pos = m.variable("Input", v2, "pos"); m.decorate(pos, "Location", 0)
    col = m.variable("Input", v4, "color"); m.decorate(col, "Location", 1)
    out = m.variable("Output", v4, "vColor"); m.decorate(out, "Location", 0)
    pv_t, pv = m.per_vertex_block()

    def body(m):
        m.store(out, m.load(v4, col))
        p = m.load(v2, pos)
        p4 = m.op("CompositeConstruct", v4, p, m.const_f(0.0), m.const_f(1.0))
        m.store(m.access("Output", v4, pv, m.const_int(0)), p4)
        m.op_void("Return")
    return m.assemble(body)


def meshpc_vert():
    """layout(push_constant) uniform PC { mat4 mvp; vec4 color; };
    layout(location=0) in vec3 pos; layout(location=1) in vec3 normal; layout(location=2) in vec4 offset;
    layout(location=0) out vec3 vN;
    void main() { vN = normal; gl_Position = mvp * vec4(pos + offset.xyz, 1.0); }"""
    m = Module(0)
    v3, v4, mat = m.vec(3), m.vec(4), m.mat4()
    pc = m.ubo_block("PC", [mat, v4], [0, 64], binding=0, sc="PushConstant")
    pos = m.variable("Input", v3, "pos"); m.decorate(pos, "Location", 0)
    nrm = m.variable("Input", v3, "normal"); m.decorate(nrm, "Location", 1)
    off = m.variable("Input", v4, "offset"); m.decorate(off, "Location", 2)
    on = m.variable("Output", v3, "vN"); m.decorate(on, "Location", 0)
    pv_t, pv = m.per_vertex_block()

    def body(m):
        m.store(on, m.load(v3, nrm))
        o = m.load(v4, off)
        oxyz = m.op("VectorShuffle", v3, o, o, 0, 1, 2)
        s = m.op("FAdd", v3, m.load(v3, pos), oxyz)
        p4 = m.op("CompositeConstruct", v4, s, m.const_f(1.0))
        mv = m.load(mat, m.access("PushConstant", mat, pc, m.const_int(0)))
        r = m.op("MatrixTimesVector", v4, mv, p4)
        m.store(m.access("Output", v4, pv, m.const_int(0)), r)
        m.op_void("Return")
    return m.assemble(body)


def meshpc_frag():
    """layout(push_constant) uniform PC { mat4 mvp; vec4 color; };
    layout(location=0) in vec3 n; layout(location=0) out vec4 o;
    void main() { float l = max(dot(normalize(n), vec3(0.48, 0.6, 0.64)), 0.0) * 0.8 + 0.2;
                  o = vec4(color.xyz * l, color.w); }"""
    m = Module(4)
    v3, v4, mat, f = m.vec(3), m.vec(4), m.mat4(), m.float()
    pc = m.ubo_block("PC", [mat, v4], [0, 64], binding=0, sc="PushConstant")
    n = m.variable("Input", v3, "n"); m.decorate(n, "Location", 0)
    out = m.variable("Output", v4, "o"); m.decorate(out, "Location", 0)
    light = m._const(("cc_light",), "ConstantComposite", lambda: v3,
                     lambda: [m.const_f(0.48), m.const_f(0.6), m.const_f(0.64)])

    def body(m):
        nn = m.ext_inst(v3, "Normalize", m.load(v3, n))
        d = m.op("Dot", f, nn, light)
        l0 = m.ext_inst(f, "FMax", d, m.const_f(0.0))
        l1 = m.op("FMul", f, l0, m.const_f(0.8))
        l = m.op("FAdd", f, l1, m.const_f(0.2))
        col = m.load(v4, m.access("PushConstant", v4, pc, m.const_int(1)))
        cxyz = m.op("VectorShuffle", v3, col, col, 0, 1, 2)
        rgb = m.op("VectorTimesScalar", v3, cxyz, l)
        cw = m.op("CompositeExtract", f, col, 3)
        m.store(out, m.op("CompositeConstruct", v4, rgb, cw))
        m.op_void("Return")
    return m.assemble(body)


def fetch_frag():
    """layout(constant_id = 0) const int K = 3; const int S = K * 8 + 8;
    layout(set=0,binding=1) uniform sampler2D tex;
    layout(location=0) in vec2 uv; layout(location=1) in vec3 n; layout(location=0) out vec4 o;
    void main() { vec4 a, b; ivec2 p = ivec2(uv * float(S));
                  a = texelFetch(tex, p, 0);       // OpImage + OpImageFetch
                  b = a;                           // OpCopyMemory
                  o = vec4(b.rgb, float(bitCount(p.x ^ p.y)) / 16.0); }"""
    m = Module(4)
    v2, v3, v4, f, i = m.vec(2), m.vec(3), m.vec(4), m.float(), m.int()
    iv2 = m.ivec(2)
    simg, img = m.sampled_image_2d(), m.image_2d()
    tex = m.variable("UniformConstant", simg, "tex")
    m.decorate(tex, "DescriptorSet", 0)
    m.decorate(tex, "Binding", 1)
    uv = m.variable("Input", v2, "uv"); m.decorate(uv, "Location", 0)
    n = m.variable("Input", v3, "n"); m.decorate(n, "Location", 1)
    out = m.variable("Output", v4, "o"); m.decorate(out, "Location", 0)
    k = m.spec_const_int(3, 0)
    scale = m.spec_op(i, "IAdd", m.spec_op(i, "IMul", k, m.const_int(8)), m.const_int(8))

    def body(m):
        a = m.local(v4)
        b = m.local(v4)
        sf = m.op("ConvertSToF", f, scale)
        p = m.op("ConvertFToS", iv2, m.op("VectorTimesScalar", v2, m.load(v2, uv), sf))
        im = m.op("Image", img, m.load(simg, tex))
        m.store(a, m.op("ImageFetch", v4, im, p, 0x2, m.const_int(0)))
        m.op_void("CopyMemory", b, a)
        g = m.load(v4, b)
        x = m.op("BitwiseXor", i, m.op("CompositeExtract", i, p, 0), m.op("CompositeExtract", i, p, 1))
        alpha = m.op("FDiv", f, m.op("ConvertSToF", f, m.op("BitCount", i, x)), m.const_f(16.0))
        rgb = m.op("VectorShuffle", v3, g, g, 0, 1, 2)
        m.store(out, m.op("CompositeConstruct", v4, rgb, alpha))
        m.op_void("Return")
    return m.assemble(body)


def storage_frag():
    """layout(set=0,binding=1,rgba8) uniform readonly image2D img;
    layout(location=0) in vec2 uv; layout(location=1) in vec3 n; layout(location=0) out vec4 o;
    void main() { o = imageLoad(img, ivec2(uv * 64.0)); }"""
    m = Module(4)
    v2, v3, v4 = m.vec(2), m.vec(3), m.vec(4)
    iv2 = m.ivec(2)
    img = m.storage_image_2d_rgba8()
    var = m.variable("UniformConstant", img, "img")
    m.decorate(var, "DescriptorSet", 0)
    m.decorate(var, "Binding", 1)
    uv = m.variable("Input", v2, "uv"); m.decorate(uv, "Location", 0)
    n = m.variable("Input", v3, "n"); m.decorate(n, "Location", 1)
    out = m.variable("Output", v4, "o"); m.decorate(out, "Location", 0)

    def body(m):
        p = m.op("ConvertFToS", iv2, m.op("VectorTimesScalar", v2, m.load(v2, uv), m.const_f(64.0)))
        m.store(out, m.op("ImageRead", v4, m.load(img, var), p))
        m.op_void("Return")
    return m.assemble(body)


def separate_frag():
    """texlit_frag with layout(set=0,binding=1) uniform texture2D t and
    layout(set=0,binding=2) uniform sampler s, sampled as texture(sampler2D(t, s), uv)."""
    m = Module(4)
    v2, v3, v4, mat, f = m.vec(2), m.vec(3), m.vec(4), m.mat4(), m.float()
    ubo = m.ubo_block("UBO", [mat, v4], [0, 64], binding=0)
    img, smp, simg = m.image_2d(), m.sampler(), m.sampled_image_2d()
    tv = m.variable("UniformConstant", img, "t")
    m.decorate(tv, "DescriptorSet", 0)
    m.decorate(tv, "Binding", 1)
    sv = m.variable("UniformConstant", smp, "s")
    m.decorate(sv, "DescriptorSet", 0)
    m.decorate(sv, "Binding", 2)
    uv = m.variable("Input", v2, "uv"); m.decorate(uv, "Location", 0)
    n = m.variable("Input", v3, "n"); m.decorate(n, "Location", 1)
    out = m.variable("Output", v4, "o"); m.decorate(out, "Location", 0)

    def body(m):
        si = m.op("SampledImage", simg, m.load(img, tv), m.load(smp, sv))
        c = m.op("ImageSampleImplicitLod", v4, si, m.load(v2, uv))
        nn = m.ext_inst(v3, "Normalize", m.load(v3, n))
        light = m.load(v4, m.access("Uniform", v4, ubo, m.const_int(1)))
        lxyz = m.op("VectorShuffle", v3, light, light, 0, 1, 2)
        d = m.op("Dot", f, nn, lxyz)
        l = m.ext_inst(f, "FMax", d, m.const_f(0.0))
        cxyz = m.op("VectorShuffle", v3, c, c, 0, 1, 2)
        rgb = m.op("VectorTimesScalar", v3, cxyz, l)
        cw = m.op("CompositeExtract", f, c, 3)
        m.store(out, m.op("CompositeConstruct", v4, rgb, cw))
        m.op_void("Return")
    return m.assemble(body)


def mathx_frag():
    """layout(location=0) in vec4 c; layout(location=0) out vec4 o;
    void main() { float z = c.a - c.a; float nan = z / z;
                  float r = nclamp(c.r * 3.0 - 1.0, 0.25, 0.75); r = nmin(nan, r); r = nmax(r, nan);
                  int i = int(c.g * 1000.0) - 500; uint u = uint(c.b * 65535.0);
                  int bits = findMSB(i) + findLSB(i) + sign(i);
                  vec3 refl = reflect(c.rgb, vec3(0.6, 0.0, 0.8));
                  o = vec4(r, float(bits) / 64.0, float(findMSB(u)) / 16.0, refl.x * 0.5 + 0.5); }
    (GLSL.std.450 NMin, NMax, NClamp, FindSMsb, FindILsb, SSign, FindUMsb, Reflect.)"""
    m = Module(4)
    v3, v4, f, i, u = m.vec(3), m.vec(4), m.float(), m.int(), m.uint()
    col = m.variable("Input", v4, "c")
    m.decorate(col, "Location", 0)
    out = m.variable("Output", v4, "o")
    m.decorate(out, "Location", 0)

    def body(m):
        c = m.load(v4, col)
        cr, cg, cb, ca = (m.op("CompositeExtract", f, c, k) for k in range(4))
        z = m.op("FSub", f, ca, ca)
        nan = m.op("FDiv", f, z, z)
        r = m.ext_inst(f, "NClamp", m.op("FSub", f, m.op("FMul", f, cr, m.const_f(3.0)), m.const_f(1.0)), m.const_f(0.25), m.const_f(0.75))
        r = m.ext_inst(f, "NMin", nan, r)
        r = m.ext_inst(f, "NMax", r, nan)
        iv = m.op("ISub", i, m.op("ConvertFToS", i, m.op("FMul", f, cg, m.const_f(1000.0))), m.const_int(500))
        uv = m.op("ConvertFToU", u, m.op("FMul", f, cb, m.const_f(65535.0)))
        bits = m.op("IAdd", i, m.op("IAdd", i, m.ext_inst(i, "FindSMsb", iv), m.ext_inst(i, "FindILsb", iv)), m.ext_inst(i, "SSign", iv))
        g = m.op("FDiv", f, m.op("ConvertSToF", f, bits), m.const_f(64.0))
        b = m.op("FDiv", f, m.op("ConvertSToF", f, m.ext_inst(i, "FindUMsb", uv)), m.const_f(16.0))
        rgb = m.op("VectorShuffle", v3, c, c, 0, 1, 2)
        nrm = m.op("CompositeConstruct", v3, m.const_f(0.6), m.const_f(0.0), m.const_f(0.8))
        refl = m.ext_inst(v3, "Reflect", rgb, nrm)
        a = m.op("FAdd", f, m.op("FMul", f, m.op("CompositeExtract", f, refl, 0), m.const_f(0.5)), m.const_f(0.5))
        m.store(out, m.op("CompositeConstruct", v4, r, g, b, a))
        m.op_void("Return")
    return m.assemble(body)


def calls_frag():
    """layout(location=0) in vec4 c; layout(location=0) out vec4 o;
    float scale(inout vec4 v, float s) { v = v * s; return v.x + s; }
    void check(vec4 v) { if (v.y > 0.45) discard; }
    void main() { vec4 t = c; float k = scale(t, 0.5); check(t); o = vec4(t.xyz, k); }
    (OpFunctionCall with a pointer and a value parameter, OpReturnValue, and a
    discard inside a called function; the functions precede main.)"""
    m = Module(4)
    v3, v4, f, b = m.vec(3), m.vec(4), m.float(), m.bool()
    col = m.variable("Input", v4, "c")
    m.decorate(col, "Location", 0)
    out = m.variable("Output", v4, "o")
    m.decorate(out, "Location", 0)
    pv4 = m.ptr("Function", v4)
    fn_scale_t = m._type(("fn", f, pv4, f), "TypeFunction", lambda: [f, pv4, f])
    fn_check_t = m._type(("fn", m.void(), v4), "TypeFunction", lambda: [m.void(), v4])

    # float scale(inout vec4 v, float s)
    scale = m.id()
    m.body.append(m._ins("Function", [f, scale, 0, fn_scale_t]))
    pv, ps = m.id(), m.id()
    m.body.append(m._ins("FunctionParameter", [pv4, pv]))
    m.body.append(m._ins("FunctionParameter", [f, ps]))
    m.label()
    mv = m.op("VectorTimesScalar", v4, m.load(v4, pv), ps)
    m.store(pv, mv)
    m.op_void("ReturnValue", m.op("FAdd", f, m.op("CompositeExtract", f, mv, 0), ps))
    m.body.append(m._ins("FunctionEnd", []))

    # void check(vec4 v)
    check = m.id()
    m.body.append(m._ins("Function", [m.void(), check, 0, fn_check_t]))
    pc = m.id()
    m.body.append(m._ins("FunctionParameter", [v4, pc]))
    m.label()
    cond = m.op("FOrdGreaterThan", b, m.op("CompositeExtract", f, pc, 1), m.const_f(0.45))
    kill_lbl, merge_lbl = m.id(), m.id()
    m.op_void("SelectionMerge", merge_lbl, 0)
    m.op_void("BranchConditional", cond, kill_lbl, merge_lbl)
    m.body.append(m._ins("Label", [kill_lbl]))
    m.op_void("Kill")
    m.body.append(m._ins("Label", [merge_lbl]))
    m.op_void("Return")
    m.body.append(m._ins("FunctionEnd", []))

    def body(m):
        t = m.local(v4)
        m.store(t, m.load(v4, col))
        k = m.op("FunctionCall", f, scale, t, m.const_f(0.5))
        tv = m.load(v4, t)
        m.op("FunctionCall", m.void(), check, tv)
        xyz = m.op("VectorShuffle", v3, tv, tv, 0, 1, 2)
        m.store(out, m.op("CompositeConstruct", v4, xyz, k))
        m.op_void("Return")
    return m.assemble(body)


def ssbo_frag():
    """layout(std430, set=0, binding=3) readonly buffer Rows { vec4 rows[]; };
    layout(location=0) in vec4 c; layout(location=0) out vec4 o;
    void main() { o = c * rows[1]; }
    (a storage buffer in SPIR-V 1.0 form: Uniform storage with BufferBlock,
    a runtime array)"""
    m = Module(4)
    v4 = m.vec(4)
    rarr = m._type(("rarr", v4), "TypeRuntimeArray", lambda: [v4])
    m.decorate(rarr, "ArrayStride", 16)
    st = m.struct("Rows", [rarr])
    m.member_decorate(st, 0, "Offset", 0)
    m.member_decorate(st, 0, "NonWritable")
    m.decorate(st, "BufferBlock")
    buf = m.variable("Uniform", st, "rows")
    m.decorate(buf, "DescriptorSet", 0)
    m.decorate(buf, "Binding", 3)
    col = m.variable("Input", v4, "c")
    m.decorate(col, "Location", 0)
    out = m.variable("Output", v4, "o")
    m.decorate(out, "Location", 0)

    def body(m):
        row = m.load(v4, m.access("Uniform", v4, buf, m.const_int(0), m.const_int(1)))
        m.store(out, m.op("FMul", v4, m.load(v4, col), row))
        m.op_void("Return")
    return m.assemble(body)


def mrt_frag():
    """layout(location=0) in vec4 c; layout(location=L) out vec4 oL (L = 0..7);
    void main() {
        o0 = c;                                        o1 = vec4(1.0 - c.rgb, c.a);
        o2 = c.zxyw;                                   o3 = c * 0.5;
        o4 = c * c;                                    o5 = c * 2.0 - vec4(1.0);
        o6 = vec4(c.x + c.y, c.y - c.z, c.z, 0.25);    o7 = c.wzyx; }
    One output per colour attachment of a subpass of up to eight."""
    m = Module(4)
    v4, v3, f = m.vec(4), m.vec(3), m.float()
    col = m.variable("Input", v4, "color")
    m.decorate(col, "Location", 0)
    outs = []
    for k in range(8):
        o = m.variable("Output", v4, "o%d" % k)
        m.decorate(o, "Location", k)
        outs.append(o)
    one3 = m._const(("cc_one3",), "ConstantComposite", lambda: v3, lambda: [m.const_f(1.0)] * 3)
    one4 = m._const(("cc_one4",), "ConstantComposite", lambda: v4, lambda: [m.const_f(1.0)] * 4)

    def body(m):
        c = m.load(v4, col)
        m.store(outs[0], c)
        rgb = m.op("VectorShuffle", v3, c, c, 0, 1, 2)
        inv = m.op("FSub", v3, one3, rgb)
        a = m.op("CompositeExtract", f, c, 3)
        m.store(outs[1], m.op("CompositeConstruct", v4, inv, a))
        m.store(outs[2], m.op("VectorShuffle", v4, c, c, 2, 0, 1, 3))
        m.store(outs[3], m.op("VectorTimesScalar", v4, c, m.const_f(0.5)))
        m.store(outs[4], m.op("FMul", v4, c, c))
        m.store(outs[5], m.op("FSub", v4, m.op("VectorTimesScalar", v4, c, m.const_f(2.0)), one4))
        x = m.op("CompositeExtract", f, c, 0)
        y = m.op("CompositeExtract", f, c, 1)
        z = m.op("CompositeExtract", f, c, 2)
        m.store(outs[6], m.op("CompositeConstruct", v4, m.op("FAdd", f, x, y), m.op("FSub", f, y, z), z, m.const_f(0.25)))
        m.store(outs[7], m.op("VectorShuffle", v4, c, c, 3, 2, 1, 0))
        m.op_void("Return")
    return m.assemble(body)


def mrti_frag():
    """layout(location=0) in vec4 c;
    layout(location=0) out vec4 o0; layout(location=1) out uvec4 o1;
    layout(location=2) out ivec4 o2; layout(location=3) out uvec4 o3;
    void main() { o0 = c; o1 = uvec4(c * 300.0); o2 = ivec4(c * 400.0 - vec4(200.0));
                  o3 = floatBitsToUint(c); }
    Integer outputs for integer colour attachments (values beyond an
    8-bit channel's range clamp; o3 carries float bit patterns)."""
    m = Module(4)
    v4, u4, i4 = m.vec(4), m.uvec(4), m.ivec(4)
    col = m.variable("Input", v4, "color")
    m.decorate(col, "Location", 0)
    outs = []
    for k, t in enumerate((v4, u4, i4, u4)):
        o = m.variable("Output", t, "o%d" % k)
        m.decorate(o, "Location", k)
        outs.append(o)
    c200 = m._const(("cc_200",), "ConstantComposite", lambda: v4, lambda: [m.const_f(200.0)] * 4)

    def body(m):
        c = m.load(v4, col)
        m.store(outs[0], c)
        m.store(outs[1], m.op("ConvertFToU", u4, m.op("VectorTimesScalar", v4, c, m.const_f(300.0))))
        m.store(outs[2], m.op("ConvertFToS", i4, m.op("FSub", v4, m.op("VectorTimesScalar", v4, c, m.const_f(400.0)), c200)))
        m.store(outs[3], m.op("Bitcast", u4, c))
        m.op_void("Return")
    return m.assemble(body)


PROGRAMS = {
    "cube": (cube_vert, lambda: colour_frag()),
    "texlit": (texlit_vert, texlit_frag),
    "flatquad": (flatquad_vert, lambda: colour_frag("Flat")),
    "meshpc": (meshpc_vert, meshpc_frag),
    "discard": (cube_vert, lambda: colour_frag(discard=True)),
    "nopersp": (cube_vert, lambda: colour_frag("NoPerspective")),
    "points": (points_vert, colour_frag),
    "fetch": (texlit_vert, fetch_frag),
    "mrt": (cube_vert, mrt_frag),
    "mrti": (cube_vert, mrti_frag),
    "storage": (texlit_vert, storage_frag),
    "separate": (texlit_vert, separate_frag),
    "mathx": (cube_vert, mathx_frag),
    "calls": (cube_vert, calls_frag),
    "ssbo": (cube_vert, ssbo_frag),
}


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name, (vert, frag) in PROGRAMS.items():
        for stage, fn in (("vert", vert), ("frag", frag)):
            with open(os.path.join(outdir, "%s.%s.spv" % (name, stage)), "wb") as fh:
                fh.write(fn())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
