// spirv.cpp — SPIR-V reader and SPIR-V → CUDA C++ translator (see spirv.h).
//
// The translation follows the semantics the reference gives each opcode in
// LLVMRuntime/SPIRVCompiler.cpp:1938-3531 (and its runtime helpers in
// CPVulkan/GlslFunctions.cpp and LLVMRuntime/SpirvFunctions.cpp), but emits
// straight-line CUDA with one explicitly rounded IEEE operation per SPIR-V
// arithmetic op (__fadd_rn & co.), so that NVRTC's -fmad=false build matches
// the reference's uncontracted binary32 arithmetic bit for bit.
//
// Structure of the emitted code for one stage:
//   * every SSA result is a local `r<id>` declared up front; every Input,
//     Output, Private and Function variable a local `v<id>`;
//   * uniform blocks and push constants are read in place through byte
//     offsets from their Offset/ArrayStride/MatrixStride decorations;
//   * blocks become labels, branches gotos, OpPhi copies on the incoming edges;
//   * OpKill returns "discarded" from the fragment function
//     (LLVMRuntime/SPIRVCompiler.cpp:3308-3310).
#include "spirv.h"

#include <cstring>
#include <functional>
#include <set>
#include <sstream>

namespace cpv::spirv {

namespace {

enum Op : uint16_t {
    OpUndef = 1, OpName = 5, OpExtInstImport = 11, OpExtInst = 12, OpMemoryModel = 14, OpEntryPoint = 15,
    OpExecutionMode = 16, OpTypeVoid = 19, OpTypeBool = 20, OpTypeInt = 21, OpTypeFloat = 22, OpTypeVector = 23,
    OpTypeMatrix = 24, OpTypeImage = 25, OpTypeSampler = 26, OpTypeSampledImage = 27, OpTypeArray = 28,
    OpTypeRuntimeArray = 29, OpTypeStruct = 30, OpTypePointer = 32, OpTypeFunction = 33, OpConstantTrue = 41,
    OpConstantFalse = 42, OpConstant = 43, OpConstantComposite = 44, OpConstantNull = 46, OpSpecConstantTrue = 48,
    OpSpecConstantFalse = 49, OpSpecConstant = 50, OpSpecConstantComposite = 51, OpFunction = 54,
    OpFunctionParameter = 55, OpFunctionEnd = 56, OpFunctionCall = 57, OpVariable = 59, OpLoad = 61, OpStore = 62,
    OpAccessChain = 65, OpInBoundsAccessChain = 66, OpDecorate = 71, OpMemberDecorate = 72,
    OpVectorExtractDynamic = 77, OpVectorInsertDynamic = 78, OpVectorShuffle = 79, OpCompositeConstruct = 80,
    OpCompositeExtract = 81, OpCompositeInsert = 82, OpCopyObject = 83, OpTranspose = 84, OpSampledImage = 86,
    OpImageSampleImplicitLod = 87, OpImageSampleExplicitLod = 88, OpConvertFToU = 109, OpConvertFToS = 110,
    OpConvertSToF = 111, OpConvertUToF = 112, OpUConvert = 113, OpSConvert = 114, OpFConvert = 115, OpBitcast = 124,
    OpSNegate = 126, OpFNegate = 127, OpIAdd = 128, OpFAdd = 129, OpISub = 130, OpFSub = 131, OpIMul = 132,
    OpFMul = 133, OpUDiv = 134, OpSDiv = 135, OpFDiv = 136, OpUMod = 137, OpSRem = 138, OpSMod = 139, OpFRem = 140,
    OpFMod = 141, OpVectorTimesScalar = 142, OpMatrixTimesScalar = 143, OpVectorTimesMatrix = 144,
    OpMatrixTimesVector = 145, OpMatrixTimesMatrix = 146, OpDot = 148, OpAny = 154, OpAll = 155, OpIsNan = 156,
    OpIsInf = 157, OpLogicalEqual = 164, OpLogicalNotEqual = 165, OpLogicalOr = 166, OpLogicalAnd = 167,
    OpLogicalNot = 168, OpSelect = 169, OpIEqual = 170, OpINotEqual = 171, OpUGreaterThan = 172,
    OpSGreaterThan = 173, OpUGreaterThanEqual = 174, OpSGreaterThanEqual = 175, OpULessThan = 176,
    OpSLessThan = 177, OpULessThanEqual = 178, OpSLessThanEqual = 179, OpFOrdEqual = 180, OpFUnordEqual = 181,
    OpFOrdNotEqual = 182, OpFUnordNotEqual = 183, OpFOrdLessThan = 184, OpFUnordLessThan = 185,
    OpFOrdGreaterThan = 186, OpFUnordGreaterThan = 187, OpFOrdLessThanEqual = 188, OpFUnordLessThanEqual = 189,
    OpFOrdGreaterThanEqual = 190, OpFUnordGreaterThanEqual = 191, OpShiftRightLogical = 194,
    OpShiftRightArithmetic = 195, OpShiftLeftLogical = 196, OpBitwiseOr = 197, OpBitwiseXor = 198,
    OpBitwiseAnd = 199, OpNot = 200, OpPhi = 245, OpLoopMerge = 246, OpSelectionMerge = 247, OpLabel = 248,
    OpBranch = 249, OpBranchConditional = 250, OpSwitch = 251, OpKill = 252, OpReturn = 253, OpReturnValue = 254,
    OpUnreachable = 255, OpCopyMemory = 63, OpImageFetch = 95, OpImage = 100, OpImageRead = 98, OpImageWrite = 99, OpBitCount = 205, OpSpecConstantOp = 52,
};

enum Dec : uint32_t {
    DecSpecId = 1, DecBlock = 2, DecBufferBlock = 3, DecRowMajor = 4, DecArrayStride = 6, DecMatrixStride = 7,
    DecBuiltIn = 11, DecNoPerspective = 13, DecFlat = 14, DecLocation = 30, DecBinding = 33, DecDescriptorSet = 34,
    DecOffset = 35,
};

enum Storage : uint32_t {
    SCUniformConstant = 0, SCInput = 1, SCUniform = 2, SCOutput = 3, SCPrivate = 6, SCFunction = 7,
    SCPushConstant = 9, SCStorageBuffer = 12,
};

enum BuiltIn : uint32_t {
    BIPosition = 0, BIPointSize = 1, BIClipDistance = 3, BICullDistance = 4, BIVertexId = 5, BIInstanceId = 6,
    BIFragCoord = 15, BIFrontFacing = 17, BIVertexIndex = 42, BIInstanceIndex = 43,
};

std::string str_from_words(const std::vector<uint32_t>& w, size_t start, size_t* consumed = nullptr) {
    std::string s;
    size_t i = start;
    for (; i < w.size(); i++) {
        const uint32_t word = w[i];
        bool end = false;
        for (int b = 0; b < 4; b++) {
            const char c = static_cast<char>((word >> (8 * b)) & 0xFF);
            if (c == 0) { end = true; break; }
            s.push_back(c);
        }
        if (end) { i++; break; }
    }
    if (consumed) *consumed = i - start;
    return s;
}

}  // namespace

bool Module::has_decoration(uint32_t id, uint32_t kind) const {
    auto it = decorations.find(id);
    if (it == decorations.end()) return false;
    for (auto& d : it->second)
        if (d.kind == kind) return true;
    return false;
}

bool Module::decoration(uint32_t id, uint32_t kind, uint32_t& value) const {
    auto it = decorations.find(id);
    if (it == decorations.end()) return false;
    for (auto& d : it->second)
        if (d.kind == kind) {
            value = d.literals.empty() ? 0 : d.literals[0];
            return true;
        }
    return false;
}

bool Module::member_decoration(uint32_t st, uint32_t member, uint32_t kind, uint32_t& value) const {
    auto it = member_decorations.find({st, member});
    if (it == member_decorations.end()) return false;
    for (auto& d : it->second)
        if (d.kind == kind) {
            value = d.literals.empty() ? 0 : d.literals[0];
            return true;
        }
    return false;
}

const EntryPoint* Module::find_entry(uint32_t model, const std::string& name) const {
    for (auto& e : entries)
        if (e.model == model && e.name == name) return &e;
    return nullptr;
}

bool parse(const uint32_t* words, size_t n, Module& m, std::string& error) {
    if (n < 5 || words[0] != 0x07230203u) {
        error = "not a SPIR-V module (bad magic)";
        return false;
    }
    m.version = words[1];
    m.bound = words[3];
    size_t i = 5;
    Function* fn = nullptr;
    Block* blk = nullptr;
    while (i < n) {
        const uint32_t w0 = words[i];
        const uint16_t op = static_cast<uint16_t>(w0 & 0xFFFF);
        const uint32_t count = w0 >> 16;
        if (count == 0 || i + count > n) {
            error = "truncated instruction";
            return false;
        }
        Instruction ins;
        ins.opcode = op;
        ins.words.assign(words + i + 1, words + i + count);
        i += count;
        const auto& w = ins.words;
        auto need = [&](size_t k) {
            if (w.size() < k) {
                error = "short operand list for opcode " + std::to_string(op);
                return false;
            }
            return true;
        };
        switch (op) {
        case OpName:
            if (!need(1)) return false;
            m.names[w[0]] = str_from_words(w, 1);
            break;
        case OpExtInstImport:
            if (!need(1)) return false;
            m.ext_imports[w[0]] = str_from_words(w, 1);
            break;
        case OpEntryPoint: {
            if (!need(3)) return false;
            EntryPoint e;
            e.model = w[0];
            e.function = w[1];
            size_t used = 0;
            e.name = str_from_words(w, 2, &used);
            for (size_t k = 2 + used; k < w.size(); k++) e.interface.push_back(w[k]);
            m.entries.push_back(e);
            break;
        }
        case OpExecutionMode:
            if (!need(2)) return false;
            m.exec_modes[w[0]].push_back(w[1]);
            break;
        case OpDecorate: {
            if (!need(2)) return false;
            Decoration d;
            d.kind = w[1];
            d.literals.assign(w.begin() + 2, w.end());
            m.decorations[w[0]].push_back(d);
            break;
        }
        case OpMemberDecorate: {
            if (!need(3)) return false;
            Decoration d;
            d.kind = w[2];
            d.literals.assign(w.begin() + 3, w.end());
            m.member_decorations[{w[0], w[1]}].push_back(d);
            break;
        }
        case OpTypeVoid: if (!need(1)) return false; m.types[w[0]].kind = TypeKind::Void; break;
        case OpTypeBool: if (!need(1)) return false; m.types[w[0]].kind = TypeKind::Bool; break;
        case OpTypeInt: {
            if (!need(3)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Int;
            t.width = w[1];
            t.is_signed = w[2] != 0;
            break;
        }
        case OpTypeFloat: {
            if (!need(2)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Float;
            t.width = w[1];
            break;
        }
        case OpTypeVector:
        case OpTypeMatrix: {
            if (!need(3)) return false;
            Type& t = m.types[w[0]];
            t.kind = op == OpTypeVector ? TypeKind::Vector : TypeKind::Matrix;
            t.component = w[1];
            t.count = w[2];
            break;
        }
        case OpTypeImage: {
            if (!need(1)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Image;
            if (w.size() >= 8) {
                t.dim = w[2];
                t.sampled = w[6];
                t.image_format = w[7];
            }
            break;
        }
        case OpTypeSampler: if (!need(1)) return false; m.types[w[0]].kind = TypeKind::Sampler; break;
        case OpTypeSampledImage: {
            if (!need(2)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::SampledImage;
            t.component = w[1];
            break;
        }
        case OpTypeArray: {
            if (!need(3)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Array;
            t.component = w[1];
            auto c = m.constants.find(w[2]);
            if (c == m.constants.end() || c->second.words.empty()) {
                error = "array length is not a constant";
                return false;
            }
            t.count = c->second.words[0];
            break;
        }
        case OpTypeRuntimeArray: {
            if (!need(2)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::RuntimeArray;
            t.component = w[1];
            break;
        }
        case OpTypeStruct: {
            if (!need(1)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Struct;
            t.members.assign(w.begin() + 1, w.end());
            break;
        }
        case OpTypePointer: {
            if (!need(3)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Pointer;
            t.storage = w[1];
            t.component = w[2];
            break;
        }
        case OpTypeFunction: {
            if (!need(2)) return false;
            Type& t = m.types[w[0]];
            t.kind = TypeKind::Function;
            t.result = w[1];
            t.members.assign(w.begin() + 2, w.end());
            break;
        }
        case OpConstantTrue:
        case OpConstantFalse:
        case OpSpecConstantTrue:
        case OpSpecConstantFalse: {
            if (!need(2)) return false;
            Constant& c = m.constants[w[1]];
            c.type = w[0];
            c.words = {(op == OpConstantTrue || op == OpSpecConstantTrue) ? 1u : 0u};
            c.spec = op == OpSpecConstantTrue || op == OpSpecConstantFalse;
            break;
        }
        case OpConstant:
        case OpSpecConstant: {
            if (!need(3)) return false;
            Constant& c = m.constants[w[1]];
            c.type = w[0];
            c.words.assign(w.begin() + 2, w.end());
            c.spec = op == OpSpecConstant;
            break;
        }
        case OpConstantComposite:
        case OpSpecConstantComposite: {
            if (!need(2)) return false;
            Constant& c = m.constants[w[1]];
            c.type = w[0];
            c.composite = true;
            c.constituents.assign(w.begin() + 2, w.end());
            break;
        }
        case OpConstantNull: {
            if (!need(2)) return false;
            Constant& c = m.constants[w[1]];
            c.type = w[0];
            c.null = true;
            break;
        }
        case OpSpecConstantOp: {
            // (result type, id, opcode, operands...): folded when the
            // module is translated (LLVMRuntime/SPIRVCompiler.cpp:938-1052)
            if (!need(4)) return false;
            Constant& c = m.constants[w[1]];
            c.type = w[0];
            c.spec_op = w[2];
            c.constituents.assign(w.begin() + 3, w.end());
            break;
        }
        case OpUndef:
            if (!need(2)) return false;
            m.undefs[w[1]] = w[0];
            break;
        case OpVariable: {
            if (!need(3)) return false;
            if (fn) {
                if (!blk) {
                    error = "variable outside a block";
                    return false;
                }
                blk->body.push_back(ins);
            } else {
                Variable v;
                v.type = w[0];
                v.id = w[1];
                v.storage = w[2];
                v.init = w.size() > 3 ? w[3] : 0;
                m.globals.push_back(v);
            }
            break;
        }
        case OpFunction: {
            if (!need(4)) return false;
            Function& f = m.functions[w[1]];
            f.id = w[1];
            f.result_type = w[0];
            f.type = w[3];
            fn = &f;
            blk = nullptr;
            break;
        }
        case OpFunctionParameter:
            if (!fn || !need(2)) { error = "parameter outside a function"; return false; }
            fn->params.push_back(w[1]);
            fn->param_types.push_back(w[0]);
            break;
        case OpFunctionEnd:
            fn = nullptr;
            blk = nullptr;
            break;
        case OpLabel:
            if (!fn || !need(1)) { error = "label outside a function"; return false; }
            fn->blocks.push_back(Block{});
            blk = &fn->blocks.back();
            blk->label = w[0];
            break;
        default:
            if (fn && blk) blk->body.push_back(ins);
            break;
        }
    }
    // Apply SpecId decorations.
    for (auto& kv : m.constants) {
        uint32_t sid;
        if (kv.second.spec && m.decoration(kv.first, DecSpecId, sid)) kv.second.spec_id = sid;
    }
    return true;
}

// ============================================================================
// Translator
// ============================================================================

namespace {

struct PtrInfo {
    // Handle: a combined image sampler (its texture slot); ImageVar /
    // SamplerVar: a separate image or sampler binding, given a slot when an
    // instruction uses it (OpSampledImage, OpImageRead, OpImageFetch)
    enum Kind { None, Lvalue, Explicit, Handle, ImageVar, SamplerVar } kind = None;
    std::string lvalue;
    std::string base, bytes, offset;  // explicit layout: byte pointer, bytes available, offset expression
    uint32_t type = 0;                // pointee type
    uint32_t mstride = 16;            // matrix stride for matrix pointees
    uint32_t slot = 0;                // handle slot
    uint32_t set = 0, binding = 0;    // ImageVar / SamplerVar descriptor
};

class Translator {
public:
    Translator(const Module& m, uint32_t model, const std::vector<SpecConstant>& spec, const std::vector<VertexBinding>& bindings,
               const std::vector<VertexAttribute>& attributes, std::vector<ResourceSlot>& slots, bool spec_lod)
        : m_(m), model_(model), spec_(spec), bindings_(bindings), attributes_(attributes), slots_(slots), spec_lod_(spec_lod && model == 4) {}

    bool run(const std::string& entry_name, StageResult& out, std::string& error);

private:
    const Module& m_;
    uint32_t model_;
    const std::vector<SpecConstant>& spec_;
    const std::vector<VertexBinding>& bindings_;
    const std::vector<VertexAttribute>& attributes_;
    std::vector<ResourceSlot>& slots_;
    bool spec_lod_;  // FS: implicit-LOD sampling takes λ from quad derivatives

    std::ostringstream types_;    // struct/array definitions
    std::ostringstream loaders_;  // explicit-layout load helpers
    std::ostringstream decls_;    // locals
    std::ostringstream pro_;      // prologue (input fetch)
    std::ostringstream body_;     // blocks
    std::ostringstream epi_;      // epilogue
    std::set<uint32_t> emitted_types_;
    std::set<uint32_t> emitted_loaders_;
    std::map<uint32_t, PtrInfo> ptrs_;
    std::map<uint32_t, uint32_t> value_type_;  // SSA id → type
    std::map<uint32_t, uint32_t> handles_;     // SSA id holding a sampled image → slot
    std::map<uint32_t, PtrInfo> images_;       // SSA id holding a separate image → its binding
    std::map<uint32_t, PtrInfo> samplers_;     // SSA id holding a sampler → its binding
    std::string err_;
    bool has_kill_ = false;
    uint32_t samples_ = 0;
    uint32_t lod_sites_ = 0;  // implicit-LOD sampling instructions (spec_lod_)
    uint32_t instructions_ = 0;
    uint32_t out_outputs_ = 0;  // FS output locations declared
    // Functions other than the entry point: each becomes a lambda inside the
    // stage function (capturing the stage's variables by reference), defined
    // callee first. While one is emitted, callee_ is it.
    std::ostringstream funcs_;
    const Function* callee_ = nullptr;
    bool emit_callee(const Function& f);
    bool order_callees(uint32_t fid, std::vector<uint32_t>& order, std::set<uint32_t>& seen, std::set<uint32_t>& stack);
    std::string callee_default_return();

    bool fail(const std::string& e) {
        if (err_.empty()) err_ = e;
        return false;
    }

    const Type* type(uint32_t id) const {
        auto it = m_.types.find(id);
        return it == m_.types.end() ? nullptr : &it->second;
    }

    bool is_float_scalar(uint32_t t) const { auto* ty = type(t); return ty && ty->kind == TypeKind::Float; }

    // ---- type names ----
    std::string tn(uint32_t id) {
        const Type* t = type(id);
        if (!t) { fail("unknown type " + std::to_string(id)); return "int"; }
        switch (t->kind) {
        case TypeKind::Void: return "void";
        case TypeKind::Bool: return "bool";
        case TypeKind::Int:
            if (t->width != 32) fail("only 32-bit integers are supported");
            return t->is_signed ? "int32_t" : "uint32_t";
        case TypeKind::Float:
            if (t->width != 32) fail("only 32-bit floats are supported");
            return "float";
        case TypeKind::Vector: return "cvec<" + tn(t->component) + ", " + std::to_string(t->count) + ">";
        case TypeKind::Matrix: {
            const Type* col = type(t->component);
            if (!col || col->kind != TypeKind::Vector) { fail("bad matrix column"); return "int"; }
            if (!is_float_scalar(col->component)) fail("only float matrices are supported");
            return "cmat<" + std::to_string(t->count) + ", " + std::to_string(col->count) + ">";
        }
        case TypeKind::Array:
            emit_aggregate(id);
            return "A" + std::to_string(id);
        case TypeKind::Struct:
            emit_aggregate(id);
            return "S" + std::to_string(id);
        case TypeKind::SampledImage:
        case TypeKind::Image:
        case TypeKind::Sampler: return "uint32_t";  /* handles: resolved at translation, never read */
        default:
            fail("unsupported type kind in shader");
            return "int";
        }
    }

    void emit_aggregate(uint32_t id) {
        if (emitted_types_.count(id)) return;
        emitted_types_.insert(id);
        const Type* t = type(id);
        if (t->kind == TypeKind::Array) {
            const std::string et = tn(t->component);
            types_ << "struct A" << id << " { " << et << " a[" << t->count << "]; };\n";
        } else {
            std::vector<std::string> mt;
            for (uint32_t mid : t->members) mt.push_back(tn(mid));
            types_ << "struct S" << id << " {";
            for (size_t i = 0; i < mt.size(); i++) types_ << " " << mt[i] << " m" << i << ";";
            types_ << " };\n";
        }
    }

    // Number of scalar components of a (float/int) type, for varying packing.
    bool flatten(uint32_t tid, const std::string& path, std::vector<std::pair<std::string, uint32_t>>& out) {
        const Type* t = type(tid);
        if (!t) return fail("bad varying type");
        switch (t->kind) {
        case TypeKind::Float:
        case TypeKind::Int:
            out.push_back({path, tid});
            return true;
        case TypeKind::Vector:
            for (uint32_t i = 0; i < t->count; i++) out.push_back({path + ".v[" + std::to_string(i) + "]", t->component});
            return true;
        case TypeKind::Matrix: {
            const Type* col = type(t->component);
            for (uint32_t c = 0; c < t->count; c++)
                for (uint32_t r = 0; r < col->count; r++)
                    out.push_back({path + ".c[" + std::to_string(c) + "].v[" + std::to_string(r) + "]", col->component});
            return true;
        }
        case TypeKind::Array:
            for (uint32_t i = 0; i < t->count; i++)
                if (!flatten(t->component, path + ".a[" + std::to_string(i) + "]", out)) return false;
            return true;
        case TypeKind::Struct:
            for (size_t i = 0; i < t->members.size(); i++)
                if (!flatten(t->members[i], path + ".m" + std::to_string(i), out)) return false;
            return true;
        default:
            return fail("unsupported varying type");
        }
    }

    // ---- constants ----
    std::string const_expr(uint32_t id) {
        auto it = m_.constants.find(id);
        if (it == m_.constants.end()) return "";
        const Constant& c = it->second;
        const Type* t = type(c.type);
        if (!t) { fail("constant of unknown type"); return "0"; }
        if (c.null) return tn(c.type) + "{}";
        if (c.spec_op) return spec_op_expr(c);
        if (c.composite) {
            // cvec/cmat/array wrappers hold one array member: double braces;
            // structs list their members: single braces.
            const bool one_array = t->kind != TypeKind::Struct;
            std::string s = tn(c.type) + (one_array ? "{{" : "{");
            for (size_t i = 0; i < c.constituents.size(); i++) {
                if (i) s += ", ";
                s += value(c.constituents[i]);
            }
            return s + (one_array ? "}}" : "}");
        }
        std::vector<uint32_t> words = c.words;
        if (c.spec && c.spec_id != 0xFFFFFFFFu) {
            for (auto& sc : spec_) {
                if (sc.id == c.spec_id && !sc.bytes.empty()) {
                    uint32_t v = 0;
                    std::memcpy(&v, sc.bytes.data(), std::min<size_t>(4, sc.bytes.size()));
                    words = {v};
                    if (t->kind == TypeKind::Bool) words = {v != 0 ? 1u : 0u};
                }
            }
        }
        const uint32_t v = words.empty() ? 0 : words[0];
        char buf[64];
        switch (t->kind) {
        case TypeKind::Bool: return v ? "true" : "false";
        case TypeKind::Int:
            if (t->is_signed) { std::snprintf(buf, sizeof(buf), "int32_t(%d)", static_cast<int32_t>(v)); return buf; }
            std::snprintf(buf, sizeof(buf), "%uu", v);
            return buf;
        case TypeKind::Float:
            std::snprintf(buf, sizeof(buf), "__uint_as_float(0x%08xu)", v);
            return buf;
        default:
            fail("unsupported constant type");
            return "0";
        }
    }

    // A specialisation-constant operation as a constant C++ expression of
    // its operands, with the arithmetic of the corresponding instruction
    // (integers wrap modulo 2^32; a zero divisor gives 0, as the
    // instructions here do).
    std::string spec_op_expr(const Constant& c) {
        const auto& o = c.constituents;
        auto a = [&](size_t i) { return i < o.size() ? "(" + value(o[i]) + ")" : std::string("0"); };
        const std::string rt = tn(c.type);
        auto u = [&](size_t i) { return "(uint32_t)" + a(i); };
        auto si = [&](size_t i) { return "(int32_t)" + a(i); };
        switch (c.spec_op) {
        case OpIAdd: return rt + "(" + u(0) + " + " + u(1) + ")";
        case OpISub: return rt + "(" + u(0) + " - " + u(1) + ")";
        case OpIMul: return rt + "(" + u(0) + " * " + u(1) + ")";
        case OpUDiv: return rt + "(" + u(1) + " == 0u ? 0u : " + u(0) + " / " + u(1) + ")";
        case OpSDiv: return rt + "(" + si(1) + " == 0 ? 0 : " + si(0) + " / " + si(1) + ")";
        case OpUMod: return rt + "(" + u(1) + " == 0u ? 0u : " + u(0) + " % " + u(1) + ")";
        case OpShiftLeftLogical: return rt + "(" + u(0) + " << (" + u(1) + " & 31u))";
        case OpShiftRightLogical: return rt + "(" + u(0) + " >> (" + u(1) + " & 31u))";
        case OpShiftRightArithmetic: return rt + "(" + si(0) + " >> (" + u(1) + " & 31u))";
        case OpBitwiseOr: return rt + "(" + u(0) + " | " + u(1) + ")";
        case OpBitwiseAnd: return rt + "(" + u(0) + " & " + u(1) + ")";
        case OpBitwiseXor: return rt + "(" + u(0) + " ^ " + u(1) + ")";
        case OpNot: return rt + "(~" + u(0) + ")";
        case OpSNegate: return rt + "(0u - " + u(0) + ")";
        case OpIEqual: return "(" + a(0) + " == " + a(1) + ")";
        case OpINotEqual: return "(" + a(0) + " != " + a(1) + ")";
        case OpULessThan: return "(" + u(0) + " < " + u(1) + ")";
        case OpSLessThan: return "(" + si(0) + " < " + si(1) + ")";
        case OpUGreaterThan: return "(" + u(0) + " > " + u(1) + ")";
        case OpSGreaterThan: return "(" + si(0) + " > " + si(1) + ")";
        case OpLogicalAnd: return "(" + a(0) + " && " + a(1) + ")";
        case OpLogicalOr: return "(" + a(0) + " || " + a(1) + ")";
        case OpLogicalNot: return "(!" + a(0) + ")";
        case OpSelect: return "(" + a(0) + " ? " + a(1) + " : " + a(2) + ")";
        case OpUConvert: case OpSConvert: return rt + "(" + a(0) + ")";
        case OpCompositeExtract:
            if (o.size() != 2) { fail("specialisation-constant extract of nested composites"); return "0"; }
            return a(0) + ".v[" + std::to_string(o[1]) + "]";
        default:
            fail("unsupported specialisation-constant operation " + std::to_string(c.spec_op));
            return "0";
        }
    }

    std::string value(uint32_t id) {
        auto it = m_.constants.find(id);
        if (it != m_.constants.end()) return const_expr(id);
        auto u = m_.undefs.find(id);
        if (u != m_.undefs.end()) return tn(u->second) + "{}";
        return "r" + std::to_string(id);
    }

    uint32_t type_of(uint32_t id) {
        auto c = m_.constants.find(id);
        if (c != m_.constants.end()) return c->second.type;
        auto u = m_.undefs.find(id);
        if (u != m_.undefs.end()) return u->second;
        auto v = value_type_.find(id);
        return v == value_type_.end() ? 0 : v->second;
    }

    // Component expression of value `id`: whole value for scalars, .v[i] for vectors.
    std::string comp(uint32_t id, uint32_t i) {
        const Type* t = type(type_of(id));
        if (t && t->kind == TypeKind::Vector) return value(id) + ".v[" + std::to_string(i) + "]";
        return value(id);
    }

    // ---- explicit-layout loads ----
    std::string loader(uint32_t tid) {
        const std::string name = "cpv_ld" + std::to_string(tid);
        if (emitted_loaders_.count(tid)) return name;
        emitted_loaders_.insert(tid);
        const Type* t = type(tid);
        std::ostringstream f;
        const std::string tname = tn(tid);
        f << "__device__ __forceinline__ " << tname << " " << name
          << "(const uint8_t* b, uint64_t n, uint64_t o, uint32_t ms) {\n  " << tname << " r;\n  (void)ms;\n";
        switch (t->kind) {
        case TypeKind::Float: f << "  r = cpv_ld_f32(b, n, o);\n"; break;
        case TypeKind::Int: f << "  r = " << (t->is_signed ? "cpv_ld_i32" : "cpv_ld_u32") << "(b, n, o);\n"; break;
        case TypeKind::Bool: f << "  r = cpv_ld_u32(b, n, o) != 0u;\n"; break;
        case TypeKind::Vector: {
            const std::string el = loader(t->component);
            for (uint32_t i = 0; i < t->count; i++) f << "  r.v[" << i << "] = " << el << "(b, n, o + " << 4 * i << "u, 0u);\n";
            break;
        }
        case TypeKind::Matrix: {
            const std::string col = loader(t->component);
            for (uint32_t i = 0; i < t->count; i++) f << "  r.c[" << i << "] = " << col << "(b, n, o + (uint64_t)ms * " << i << "u, 0u);\n";
            break;
        }
        case TypeKind::Array: {
            uint32_t stride = 0;
            if (!m_.decoration(tid, DecArrayStride, stride)) fail("uniform array without ArrayStride");
            const std::string el = loader(t->component);
            f << "  for (uint32_t i = 0; i < " << t->count << "u; i++) r.a[i] = " << el << "(b, n, o + (uint64_t)i * " << stride
              << "u, ms);\n";
            break;
        }
        case TypeKind::Struct: {
            for (size_t i = 0; i < t->members.size(); i++) {
                uint32_t off = 0, ms = 16;
                if (!m_.member_decoration(tid, static_cast<uint32_t>(i), DecOffset, off)) fail("uniform member without Offset");
                m_.member_decoration(tid, static_cast<uint32_t>(i), DecMatrixStride, ms);
                uint32_t rm;
                if (m_.member_decoration(tid, static_cast<uint32_t>(i), DecRowMajor, rm)) fail("row-major uniform matrices are not supported");
                f << "  r.m" << i << " = " << loader(t->members[i]) << "(b, n, o + " << off << "u, " << ms << "u);\n";
            }
            break;
        }
        default:
            fail("unsupported type in a uniform block");
            break;
        }
        f << "  return r;\n}\n";
        loaders_ << f.str();
        return name;
    }

    uint32_t slot_for(uint32_t set, uint32_t binding, bool texture) {
        for (auto& s : slots_)
            if (s.set == set && s.binding == binding && s.is_texture == texture && !s.separate) return s.slot;
        uint32_t next = 0;
        for (auto& s : slots_)
            if (s.is_texture == texture) next++;
        ResourceSlot rs;
        rs.set = set;
        rs.binding = binding;
        rs.is_texture = texture;
        rs.slot = next;
        slots_.push_back(rs);
        return next;
    }
    // the texture slot of a (sampled image, sampler) pair joined by OpSampledImage
    uint32_t slot_for_pair(const PtrInfo& image, const PtrInfo& sampler) {
        for (auto& s : slots_)
            if (s.is_texture && s.separate && s.set == image.set && s.binding == image.binding && s.sampler_set == sampler.set &&
                s.sampler_binding == sampler.binding)
                return s.slot;
        uint32_t next = 0;
        for (auto& s : slots_)
            if (s.is_texture) next++;
        ResourceSlot rs;
        rs.set = image.set;
        rs.binding = image.binding;
        rs.is_texture = true;
        rs.separate = true;
        rs.sampler_set = sampler.set;
        rs.sampler_binding = sampler.binding;
        rs.slot = next;
        slots_.push_back(rs);
        return next;
    }

    const VertexAttribute* find_attribute(uint32_t location) const {
        for (auto& a : attributes_)
            if (a.location == location) return &a;
        return nullptr;
    }
    const VertexBinding* find_binding(uint32_t binding) const {
        for (auto& b : bindings_)
            if (b.binding == binding) return &b;
        return nullptr;
    }

    bool emit_globals(const EntryPoint& ep, StageResult& out);
    bool emit_attribute_fetch(const Variable& v, uint32_t location);
    bool emit_function(const Function& f);
    bool emit_instruction(const Instruction& ins, const std::map<uint32_t, std::vector<std::string>>& phi_copies, uint32_t block);
    void cw(uint32_t rid, uint32_t rtype, const std::vector<uint32_t>& ops, const std::function<std::string(const std::vector<std::string>&)>& f);
    std::string access_lvalue(const std::string& base, uint32_t& tid, const std::vector<uint32_t>& idx_ids);
};

void Translator::cw(uint32_t rid, uint32_t rtype, const std::vector<uint32_t>& ops,
                    const std::function<std::string(const std::vector<std::string>&)>& f) {
    const Type* t = type(rtype);
    const std::string r = "r" + std::to_string(rid);
    if (t && t->kind == TypeKind::Vector) {
        for (uint32_t i = 0; i < t->count; i++) {
            std::vector<std::string> cs;
            for (uint32_t o : ops) cs.push_back(comp(o, i));
            body_ << "  " << r << ".v[" << i << "] = " << f(cs) << ";\n";
        }
    } else {
        std::vector<std::string> cs;
        for (uint32_t o : ops) cs.push_back(value(o));
        body_ << "  " << r << " = " << f(cs) << ";\n";
    }
}

std::string Translator::access_lvalue(const std::string& base, uint32_t& tid, const std::vector<uint32_t>& idx_ids) {
    std::string s = base;
    for (uint32_t idx : idx_ids) {
        const Type* t = type(tid);
        if (!t) { fail("access into unknown type"); return s; }
        switch (t->kind) {
        case TypeKind::Struct: {
            auto c = m_.constants.find(idx);
            if (c == m_.constants.end()) { fail("struct index is not constant"); return s; }
            const uint32_t k = c->second.words[0];
            s += ".m" + std::to_string(k);
            tid = t->members[k];
            break;
        }
        case TypeKind::Array: s += ".a[" + value(idx) + "]"; tid = t->component; break;
        case TypeKind::Matrix: s += ".c[" + value(idx) + "]"; tid = t->component; break;
        case TypeKind::Vector: s += ".v[" + value(idx) + "]"; tid = t->component; break;
        default: fail("bad access chain"); return s;
        }
    }
    return s;
}

bool Translator::emit_attribute_fetch(const Variable& v, uint32_t location) {
    const uint32_t tid = type(v.type)->component;
    const Type* t = type(tid);
    uint32_t comps = 0, elem = tid;
    if (t->kind == TypeKind::Vector) { comps = t->count; elem = t->component; }
    else if (t->kind == TypeKind::Float || t->kind == TypeKind::Int) comps = 1;
    else return fail("vertex input of unsupported type (location " + std::to_string(location) + ")");
    const bool is_float = is_float_scalar(elem);
    const std::string var = "v" + std::to_string(v.id);
    auto path = [&](uint32_t i) { return t->kind == TypeKind::Vector ? var + ".v[" + std::to_string(i) + "]" : var; };
    // Defaults for components the format does not provide: (0, 0, 0, 1).
    for (uint32_t i = 0; i < comps; i++) {
        if (is_float) pro_ << "  " << path(i) << " = " << (i == 3 ? "1.0f" : "0.0f") << ";\n";
        else pro_ << "  " << path(i) << " = " << (i == 3 ? "1" : "0") << ";\n";
    }
    const VertexAttribute* a = find_attribute(location);
    if (!a) return true;  // unbound input reads the defaults
    const VertexBinding* b = find_binding(a->binding);
    if (!b) return fail("vertex attribute references an undeclared binding");
    if (a->binding >= 8) return fail("vertex binding index above 7");
    uint32_t fcomps = 0, esize = 0;
    bool sgn = false, bgra = false;
    int kind = 0;  // 0 float32, 1 uint32, 2 sint32, 3 normalised 8/16-bit, 4 float16
    switch (a->format) {
    case 100: fcomps = 1; break;
    case 103: fcomps = 2; break;
    case 106: fcomps = 3; break;
    case 109: fcomps = 4; break;
    case 98: fcomps = 1; kind = 1; break;
    case 101: fcomps = 2; kind = 1; break;
    case 104: fcomps = 3; kind = 1; break;
    case 107: fcomps = 4; kind = 1; break;
    case 99: fcomps = 1; kind = 2; break;
    case 102: fcomps = 2; kind = 2; break;
    case 105: fcomps = 3; kind = 2; break;
    case 108: fcomps = 4; kind = 2; break;
    // UNORM / SNORM through the reference's pixel decoder
    // (LLVMRuntime/PipelineCompiler.cpp:855-889, CPVulkanBase/Formats.cpp)
    case 9: fcomps = 1; kind = 3; esize = 1; break;                // R8_UNORM
    case 10: fcomps = 1; kind = 3; esize = 1; sgn = true; break;   // R8_SNORM
    case 16: fcomps = 2; kind = 3; esize = 1; break;               // R8G8_UNORM
    case 17: fcomps = 2; kind = 3; esize = 1; sgn = true; break;   // R8G8_SNORM
    case 23: fcomps = 3; kind = 3; esize = 1; break;               // R8G8B8_UNORM
    case 24: fcomps = 3; kind = 3; esize = 1; sgn = true; break;   // R8G8B8_SNORM
    case 37: fcomps = 4; kind = 3; esize = 1; break;               // R8G8B8A8_UNORM
    case 38: fcomps = 4; kind = 3; esize = 1; sgn = true; break;   // R8G8B8A8_SNORM
    case 44: fcomps = 4; kind = 3; esize = 1; bgra = true; break;  // B8G8R8A8_UNORM (red in byte 2)
    case 70: fcomps = 1; kind = 3; esize = 2; break;               // R16_UNORM
    case 71: fcomps = 1; kind = 3; esize = 2; sgn = true; break;   // R16_SNORM
    case 77: fcomps = 2; kind = 3; esize = 2; break;               // R16G16_UNORM
    case 78: fcomps = 2; kind = 3; esize = 2; sgn = true; break;   // R16G16_SNORM
    case 84: fcomps = 3; kind = 3; esize = 2; break;               // R16G16B16_UNORM
    case 85: fcomps = 3; kind = 3; esize = 2; sgn = true; break;   // R16G16B16_SNORM
    case 91: fcomps = 4; kind = 3; esize = 2; break;               // R16G16B16A16_UNORM
    case 92: fcomps = 4; kind = 3; esize = 2; sgn = true; break;   // R16G16B16A16_SNORM
    // half floats: loaded as the type itself and widened (fpext), which the
    // reference does only for an input of the same width (:845-851, 711-764)
    case 76: fcomps = 1; kind = 4; esize = 2; break;   // R16_SFLOAT
    case 83: fcomps = 2; kind = 4; esize = 2; break;   // R16G16_SFLOAT
    case 90: fcomps = 3; kind = 4; esize = 2; break;   // R16G16B16_SFLOAT
    case 97: fcomps = 4; kind = 4; esize = 2; break;   // R16G16B16A16_SFLOAT
    default: return fail("unsupported vertex attribute format " + std::to_string(a->format));
    }
    if (kind == 3 && !is_float) return fail("normalised vertex attribute into an integer input (the reference aborts on it)");
    if (kind == 4 && (!is_float || fcomps != comps))
        return fail("half-float vertex attribute into an input of another type or width (the reference aborts on it)");
    const std::string index = b->input_rate == 0 ? "cpv_vertex_index" : "cpv_instance_index";
    pro_ << "  { const uint64_t off = (uint64_t)" << b->stride << "u * (uint64_t)" << index << " + " << a->offset << "u;\n";
    const uint32_t nload = comps < fcomps ? comps : fcomps;
    if (kind <= 2 && nload > 1) {
        // 32-bit channels: one bounds check for all of them (each channel's
        // own check passes exactly when the last one's does), then plain
        // loads; otherwise the per-channel checked loads below
        const std::string bs = std::to_string(a->binding);
        pro_ << "    if (P.vb[" << bs << "] != nullptr && off + " << 4 * nload << "u <= P.vb_bytes[" << bs << "]) {\n";
        pro_ << "      const uint32_t* cpv_q = reinterpret_cast<const uint32_t*>(P.vb[" << bs << "] + off);\n";
        for (uint32_t i = 0; i < nload; i++) {
            std::string e = "cpv_q[" + std::to_string(i) + "]";
            if (kind == 0) e = is_float ? "__uint_as_float(" + e + ")" : "(" + tn(elem) + ")" + e;
            else e = is_float ? "__uint_as_float(" + e + ")" : "(" + tn(elem) + ")(" + e + ")";
            pro_ << "      " << path(i) << " = " << e << ";\n";
        }
        pro_ << "    } else {\n";
    }
    for (uint32_t i = 0; i < comps && i < fcomps; i++) {
        std::string e;
        const std::string vb = "P.vb[" + std::to_string(a->binding) + "], P.vb_bytes[" + std::to_string(a->binding) + "]";
        if (kind == 3) {
            const uint32_t ch = bgra && i < 3 ? 2 - i : i;
            e = "cpv_decode_norm(cpv_ld_elem(" + vb + ", off + " + std::to_string(ch * esize) + "u, " + std::to_string(esize) + "u), " +
                std::to_string(esize) + "u, " + (sgn ? "true" : "false") + ")";
        } else if (kind == 4) {
            e = "cpv_half_to_float(cpv_ld_elem(" + vb + ", off + " + std::to_string(2 * i) + "u, 2u))";
        } else if (kind == 0) {
            e = "cpv_ld_f32(" + vb + ", off + " + std::to_string(4 * i) + "u)";
            if (!is_float) e = "(" + tn(elem) + ")__float_as_uint(" + e + ")";
        } else {
            e = "cpv_ld_u32(" + vb + ", off + " + std::to_string(4 * i) + "u)";
            e = is_float ? "__uint_as_float(" + e + ")" : "(" + tn(elem) + ")(" + e + ")";
        }
        pro_ << "    " << path(i) << " = " << e << ";\n";
    }
    if (kind <= 2 && nload > 1) pro_ << "    }\n";
    pro_ << "  }\n";
    return true;
}

bool Translator::emit_globals(const EntryPoint& ep, StageResult& out) {
    uint32_t var_floats = 0;
    (void)ep;
    for (const Variable& v : m_.globals) {
        const Type* pt = type(v.type);
        if (!pt || pt->kind != TypeKind::Pointer) return fail("global variable is not a pointer");
        const uint32_t tid = pt->component;
        const std::string var = "v" + std::to_string(v.id);
        PtrInfo info;
        info.type = tid;
        switch (v.storage) {
        case SCInput:
        case SCOutput:
        case SCPrivate: {
            decls_ << "  " << tn(tid) << " " << var << ";\n";
            if (v.init) pro_ << "  " << var << " = " << value(v.init) << ";\n";
            info.kind = PtrInfo::Lvalue;
            info.lvalue = var;
            ptrs_[v.id] = info;
            uint32_t builtin = 0, location = 0;
            const bool is_builtin = m_.decoration(v.id, DecBuiltIn, builtin);
            const bool has_location = m_.decoration(v.id, DecLocation, location);
            if (v.storage == SCInput) {
                if (model_ == 0) {
                    if (is_builtin) {
                        if (builtin == BIVertexIndex || builtin == BIVertexId) pro_ << "  " << var << " = (" << tn(tid) << ")cpv_vertex_index;\n";
                        else if (builtin == BIInstanceIndex || builtin == BIInstanceId) pro_ << "  " << var << " = (" << tn(tid) << ")cpv_instance_index;\n";
                        else return fail("unsupported vertex input builtin " + std::to_string(builtin));
                    } else if (has_location) {
                        if (!emit_attribute_fetch(v, location)) return false;
                    }
                } else {
                    if (is_builtin) {
                        if (builtin == BIFragCoord) {
                            for (int i = 0; i < 4; i++) pro_ << "  " << var << ".v[" << i << "] = cpv_frag_coord[" << i << "];\n";
                            out.reads_frag_coord = true;
                        } else if (builtin == BIFrontFacing) {
                            pro_ << "  " << var << " = cpv_front;\n";
                            out.reads_front_facing = true;
                        } else {
                            return fail("unsupported fragment input builtin " + std::to_string(builtin));
                        }
                    } else if (has_location) {
                        // CPVulkan/CommandBuffer.Draw.cpp:429-470: inputs are packed in
                        // declaration order; interpolation from the variable's decoration.
                        int interp = 0;
                        if (m_.has_decoration(v.id, DecNoPerspective)) interp = 1;
                        if (m_.has_decoration(v.id, DecFlat)) interp = 2;
                        std::vector<std::pair<std::string, uint32_t>> comps;
                        if (!flatten(tid, var, comps)) return false;
                        for (auto& c : comps) {
                            const bool fl = is_float_scalar(c.second);
                            if (!fl && interp != 2) return fail("integer fragment input without Flat");
                            pro_ << "  " << c.first << " = " << (fl ? "" : "(" + tn(c.second) + ")__float_as_uint(") << "cpv_in["
                                 << var_floats << "]" << (fl ? "" : ")") << ";\n";
                            out.interp.push_back(interp);
                            var_floats++;
                        }
                    }
                }
            } else if (v.storage == SCOutput) {
                if (model_ == 0) {
                    if (is_builtin) {
                        if (builtin == BIPosition)
                            for (int i = 0; i < 4; i++) epi_ << "  cpv_pos[" << i << "] = " << var << ".v[" << i << "];\n";
                        else if (builtin == BIPointSize) {
                            // A shader that never writes gl_PointSize gives points of size 1.
                            pro_ << "  " << var << " = 1.0f;\n";
                            epi_ << "  if (cpv_point_size) *cpv_point_size = " << var << ";\n";
                        }
                    } else if (type(tid)->kind == TypeKind::Struct && m_.has_decoration(tid, DecBlock)) {
                        const Type* st = type(tid);
                        for (size_t k = 0; k < st->members.size(); k++) {
                            uint32_t bi = 0;
                            if (!m_.member_decoration(tid, static_cast<uint32_t>(k), DecBuiltIn, bi)) continue;
                            if (bi == BIPosition)
                                for (int i = 0; i < 4; i++) epi_ << "  cpv_pos[" << i << "] = " << var << ".m" << k << ".v[" << i << "];\n";
                            else if (bi == BIPointSize) {
                                pro_ << "  " << var << ".m" << k << " = 1.0f;\n";
                                epi_ << "  if (cpv_point_size) *cpv_point_size = " << var << ".m" << k << ";\n";
                            }
                        }
                    } else if (has_location) {
                        // PipelineCompiler.cpp:957-980: outputs stored in declaration order.
                        std::vector<std::pair<std::string, uint32_t>> comps;
                        if (!flatten(tid, var, comps)) return false;
                        for (auto& c : comps) {
                            if (var_floats >= 16) return fail("more than 16 varying components");
                            const bool fl = is_float_scalar(c.second);
                            epi_ << "  cpv_var[" << var_floats << "] = " << (fl ? c.first : "__uint_as_float((uint32_t)" + c.first + ")") << ";\n";
                            var_floats++;
                        }
                    }
                } else {
                    if (is_builtin) return fail("unsupported fragment output builtin " + std::to_string(builtin));
                    if (has_location) {
                        // output L feeds colour attachment L of the subpass
                        // (LLVMRuntime/PipelineCompiler.cpp:1415-1429, 1655-1667);
                        // outputs beyond the module's attachments are dropped
                        if (location >= 8) return fail("fragment output location beyond the 8 colour attachments");
                        // a vec4, ivec4 or uvec4: an integer output's bits pass
                        // unchanged (the attachment's encoder reads them as the
                        // output's memory, :1528-1653)
                        const Type* t = type(tid);
                        const Type* ct = t ? type(t->component) : nullptr;
                        const bool int_out = ct && ct->kind == TypeKind::Int && ct->width == 32;
                        if (!t || t->kind != TypeKind::Vector || t->count != 4 || !(is_float_scalar(t->component) || int_out))
                            return fail("fragment output " + std::to_string(location) + " must be a vec4, ivec4 or uvec4");
                        if (location > 0) epi_ << "#if CPV_NUM_CA > " << location << "\n";
                        for (int i = 0; i < 4; i++) {
                            const std::string v = var + ".v[" + std::to_string(i) + "]";
                            epi_ << "  cpv_colour[" << 4 * location + i << "] = " << (int_out ? "__uint_as_float((uint32_t)" + v + ")" : v) << ";\n";
                        }
                        if (location > 0) epi_ << "#endif\n";
                        out_outputs_ |= 1u << location;
                    }
                }
            }
            break;
        }
        case SCUniform:
        case SCStorageBuffer:
        case SCPushConstant: {
            // Storage buffers (StorageBuffer, or Uniform with BufferBlock) are
            // read like uniform buffers, with explicit layout and bounds-checked
            // loads (CPVulkan/CommandBuffer.Draw.cpp:379-395 binds both alike);
            // stores through an explicit-layout pointer are rejected as writes
            // to read-only memory: fragments run concurrently here and Vulkan
            // leaves the order of their buffer writes undefined.
            info.kind = PtrInfo::Explicit;
            info.offset = "0ull";
            if (v.storage == SCPushConstant) {
                info.base = "reinterpret_cast<const uint8_t*>(P.push)";
                info.bytes = "128ull";
            } else {
                uint32_t set = 0, binding = 0;
                m_.decoration(v.id, DecDescriptorSet, set);
                m_.decoration(v.id, DecBinding, binding);
                const uint32_t s = slot_for(set, binding, false);
                if (s >= 8) return fail("more than 8 uniform buffers");
                info.base = "P.ubo[" + std::to_string(s) + "]";
                info.bytes = "P.ubo_bytes[" + std::to_string(s) + "]";
            }
            ptrs_[v.id] = info;
            break;
        }
        case SCUniformConstant: {
            const Type* t = type(tid);
            uint32_t set = 0, binding = 0;
            m_.decoration(v.id, DecDescriptorSet, set);
            m_.decoration(v.id, DecBinding, binding);
            if (t && t->kind == TypeKind::SampledImage) {
                info.kind = PtrInfo::Handle;
                info.slot = slot_for(set, binding, true);
                if (info.slot >= 4) return fail("more than 4 sampled images");
            } else if (t && t->kind == TypeKind::Image) {
                // a separate sampled image or a storage image
                // (CPVulkan/CommandBuffer.Draw.cpp:368-377): 2D only
                if (t->dim != 1) return fail("only 2D images are supported");
                info.kind = PtrInfo::ImageVar;
            } else if (t && t->kind == TypeKind::Sampler) {
                info.kind = PtrInfo::SamplerVar;
            } else {
                return fail("unsupported UniformConstant variable");
            }
            info.set = set;
            info.binding = binding;
            ptrs_[v.id] = info;
            break;
        }
        default:
            return fail("unsupported storage class " + std::to_string(v.storage));
        }
    }
    out.num_floats = var_floats;
    return true;
}

bool Translator::emit_function(const Function& f) {
    for (const Block& b : f.blocks) instructions_ += static_cast<uint32_t>(b.body.size());
    // Result types of every instruction, and function-local variables.
    for (const Block& b : f.blocks) {
        for (const Instruction& ins : b.body) {
            const auto& w = ins.words;
            if (ins.opcode == OpVariable) {
                const Type* pt = type(w[0]);
                if (!pt) return fail("bad local variable type");
                const std::string var = "v" + std::to_string(w[1]);
                decls_ << "  " << tn(pt->component) << " " << var << ";\n";
                PtrInfo info;
                info.kind = PtrInfo::Lvalue;
                info.lvalue = var;
                info.type = pt->component;
                ptrs_[w[1]] = info;
                if (w.size() > 3) pro_ << "  " << var << " = " << value(w[3]) << ";\n";
                continue;
            }
            // Instructions with a result type/result id pair.
            switch (ins.opcode) {
            case OpStore: case OpSelectionMerge: case OpLoopMerge: case OpBranch: case OpBranchConditional: case OpSwitch:
            case OpKill: case OpReturn: case OpReturnValue: case OpUnreachable:
                break;
            case OpAccessChain: case OpInBoundsAccessChain:
                break;  // pointers are resolved at translation time
            default:
                if (w.size() >= 2) {
                    const Type* rt = type(w[0]);
                    if (rt && rt->kind != TypeKind::Void && rt->kind != TypeKind::Pointer) {
                        value_type_[w[1]] = w[0];
                        if (rt->kind == TypeKind::SampledImage) break;
                        decls_ << "  " << tn(w[0]) << " r" << w[1] << ";\n";
                    }
                }
                break;
            }
        }
    }
    // Phi copies on incoming edges.
    std::map<uint32_t, std::vector<std::string>> phi_copies;  // predecessor label → statements
    for (const Block& b : f.blocks) {
        for (const Instruction& ins : b.body) {
            if (ins.opcode != OpPhi) continue;
            const auto& w = ins.words;
            decls_ << "  " << tn(w[0]) << " phi" << w[1] << ";\n";
            for (size_t k = 2; k + 1 < w.size(); k += 2)
                phi_copies[w[k + 1]].push_back("phi" + std::to_string(w[1]) + " = " + value(w[k]) + ";");
        }
    }
    for (size_t bi = 0; bi < f.blocks.size(); bi++) {
        const Block& b = f.blocks[bi];
        body_ << " L" << b.label << ":;\n";
        for (const Instruction& ins : b.body)
            if (!emit_instruction(ins, phi_copies, b.label)) return false;
    }
    return err_.empty();
}

bool Translator::emit_instruction(const Instruction& ins, const std::map<uint32_t, std::vector<std::string>>& phi_copies, uint32_t block) {
    const auto& w = ins.words;
    auto edge_copies = [&]() {
        auto it = phi_copies.find(block);
        if (it != phi_copies.end())
            for (auto& s : it->second) body_ << "  " << s << "\n";
    };
    auto R = [&](uint32_t id) { return "r" + std::to_string(id); };
    switch (ins.opcode) {
    case OpVariable:
    case OpSelectionMerge:
    case OpLoopMerge:
    case 8:   /* OpLine */
    case 317: /* OpNoLine */
    case 0:   /* OpNop */
        return true;
    case OpPhi:
        body_ << "  " << R(w[1]) << " = phi" << w[1] << ";\n";
        return true;
    case OpLoad: {
        auto it = ptrs_.find(w[2]);
        if (it == ptrs_.end()) return fail("load through an unknown pointer");
        const PtrInfo& p = it->second;
        if (p.kind == PtrInfo::Handle) {
            handles_[w[1]] = p.slot;
            return true;
        }
        if (p.kind == PtrInfo::ImageVar) {
            images_[w[1]] = p;
            return true;
        }
        if (p.kind == PtrInfo::SamplerVar) {
            samplers_[w[1]] = p;
            return true;
        }
        if (p.kind == PtrInfo::Lvalue) body_ << "  " << R(w[1]) << " = " << p.lvalue << ";\n";
        else body_ << "  " << R(w[1]) << " = " << loader(p.type) << "(" << p.base << ", " << p.bytes << ", " << p.offset << ", " << p.mstride << "u);\n";
        return true;
    }
    case OpStore: {
        auto it = ptrs_.find(w[0]);
        if (it == ptrs_.end()) return fail("store through an unknown pointer");
        if (it->second.kind != PtrInfo::Lvalue) return fail("store to read-only memory");
        body_ << "  " << it->second.lvalue << " = " << value(w[1]) << ";\n";
        return true;
    }
    case OpAccessChain:
    case OpInBoundsAccessChain: {
        auto it = ptrs_.find(w[2]);
        if (it == ptrs_.end()) return fail("access chain on an unknown pointer");
        PtrInfo p = it->second;
        std::vector<uint32_t> idx(w.begin() + 3, w.end());
        if (p.kind == PtrInfo::Lvalue) {
            uint32_t tid = p.type;
            p.lvalue = access_lvalue(p.lvalue, tid, idx);
            p.type = tid;
        } else if (p.kind == PtrInfo::Explicit) {
            uint32_t tid = p.type;
            for (uint32_t ix : idx) {
                const Type* t = type(tid);
                switch (t->kind) {
                case TypeKind::Struct: {
                    auto c = m_.constants.find(ix);
                    if (c == m_.constants.end()) return fail("struct index is not constant");
                    const uint32_t k = c->second.words[0];
                    uint32_t off = 0, ms = 16;
                    if (!m_.member_decoration(tid, k, DecOffset, off)) return fail("uniform member without Offset");
                    m_.member_decoration(tid, k, DecMatrixStride, ms);
                    p.offset = "(" + p.offset + " + " + std::to_string(off) + "ull)";
                    p.mstride = ms;
                    tid = t->members[k];
                    break;
                }
                case TypeKind::Array:
                case TypeKind::RuntimeArray: {
                    uint32_t stride = 0;
                    if (!m_.decoration(tid, DecArrayStride, stride)) return fail("uniform array without ArrayStride");
                    p.offset = "(" + p.offset + " + (uint64_t)(" + value(ix) + ") * " + std::to_string(stride) + "ull)";
                    tid = t->component;
                    break;
                }
                case TypeKind::Matrix:
                    p.offset = "(" + p.offset + " + (uint64_t)(" + value(ix) + ") * " + std::to_string(p.mstride) + "ull)";
                    tid = t->component;
                    break;
                case TypeKind::Vector:
                    p.offset = "(" + p.offset + " + (uint64_t)(" + value(ix) + ") * 4ull)";
                    tid = t->component;
                    break;
                default:
                    return fail("bad uniform access chain");
                }
            }
            p.type = tid;
        } else {
            return fail("access chain into an image handle");
        }
        ptrs_[w[1]] = p;
        return true;
    }
    case OpCopyObject:
        body_ << "  " << R(w[1]) << " = " << value(w[2]) << ";\n";
        return true;
    case OpCompositeConstruct: {
        const Type* t = type(w[0]);
        if (t->kind == TypeKind::Vector) {
            uint32_t k = 0;
            for (size_t i = 2; i < w.size(); i++) {
                const Type* ct = type(type_of(w[i]));
                if (ct && ct->kind == TypeKind::Vector) {
                    for (uint32_t j = 0; j < ct->count; j++) body_ << "  " << R(w[1]) << ".v[" << k++ << "] = " << comp(w[i], j) << ";\n";
                } else {
                    body_ << "  " << R(w[1]) << ".v[" << k++ << "] = " << value(w[i]) << ";\n";
                }
            }
        } else if (t->kind == TypeKind::Matrix) {
            for (size_t i = 2; i < w.size(); i++) body_ << "  " << R(w[1]) << ".c[" << i - 2 << "] = " << value(w[i]) << ";\n";
        } else if (t->kind == TypeKind::Array) {
            for (size_t i = 2; i < w.size(); i++) body_ << "  " << R(w[1]) << ".a[" << i - 2 << "] = " << value(w[i]) << ";\n";
        } else if (t->kind == TypeKind::Struct) {
            for (size_t i = 2; i < w.size(); i++) body_ << "  " << R(w[1]) << ".m" << i - 2 << " = " << value(w[i]) << ";\n";
        } else {
            return fail("composite construct of a scalar");
        }
        return true;
    }
    case OpCompositeExtract:
    case OpCompositeInsert: {
        const bool insert = ins.opcode == OpCompositeInsert;
        const uint32_t src = insert ? w[3] : w[2];
        uint32_t tid = type_of(src);
        std::string path = insert ? R(w[1]) : value(src);
        for (size_t i = insert ? 4 : 3; i < w.size(); i++) {
            const Type* t = type(tid);
            const uint32_t k = w[i];
            switch (t->kind) {
            case TypeKind::Vector: path += ".v[" + std::to_string(k) + "]"; tid = t->component; break;
            case TypeKind::Matrix: path += ".c[" + std::to_string(k) + "]"; tid = t->component; break;
            case TypeKind::Array: path += ".a[" + std::to_string(k) + "]"; tid = t->component; break;
            case TypeKind::Struct: path += ".m" + std::to_string(k); tid = t->members[k]; break;
            default: return fail("bad composite index");
            }
        }
        if (insert) {
            body_ << "  " << R(w[1]) << " = " << value(src) << ";\n";
            body_ << "  " << path << " = " << value(w[2]) << ";\n";
        } else {
            body_ << "  " << R(w[1]) << " = " << path << ";\n";
        }
        return true;
    }
    case OpVectorShuffle: {
        const Type* a = type(type_of(w[2]));
        const uint32_t na = a->count;
        for (size_t i = 4; i < w.size(); i++) {
            const uint32_t s = w[i];
            std::string e;
            if (s == 0xFFFFFFFFu) e = "0";
            else if (s < na) e = comp(w[2], s);
            else e = comp(w[3], s - na);
            body_ << "  " << R(w[1]) << ".v[" << i - 4 << "] = " << e << ";\n";
        }
        return true;
    }
    case OpVectorExtractDynamic:
        body_ << "  " << R(w[1]) << " = " << value(w[2]) << ".v[" << value(w[3]) << "];\n";
        return true;
    case OpVectorInsertDynamic:
        body_ << "  " << R(w[1]) << " = " << value(w[2]) << ";\n  " << R(w[1]) << ".v[" << value(w[4]) << "] = " << value(w[3]) << ";\n";
        return true;
    // ---- arithmetic ----
    case OpFAdd: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "__fadd_rn(" + c[0] + ", " + c[1] + ")"; }); return true;
    case OpFSub: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "__fsub_rn(" + c[0] + ", " + c[1] + ")"; }); return true;
    case OpFMul: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "__fmul_rn(" + c[0] + ", " + c[1] + ")"; }); return true;
    case OpFDiv: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "__fdiv_rn(" + c[0] + ", " + c[1] + ")"; }); return true;
    case OpFRem: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "fmodf(" + c[0] + ", " + c[1] + ")"; }); return true;
    case OpFMod:
        cw(w[1], w[0], {w[2], w[3]}, [](auto& c) {
            return "__fsub_rn(" + c[0] + ", __fmul_rn(" + c[1] + ", floorf(__fdiv_rn(" + c[0] + ", " + c[1] + "))))";
        });
        return true;
    case OpFNegate: cw(w[1], w[0], {w[2]}, [](auto& c) { return "(-" + c[0] + ")"; }); return true;
    case OpSNegate: cw(w[1], w[0], {w[2]}, [](auto& c) { return "(int32_t)(0u - (uint32_t)" + c[0] + ")"; }); return true;
    case OpIAdd: case OpISub: case OpIMul: {
        const char* op = ins.opcode == OpIAdd ? " + " : (ins.opcode == OpISub ? " - " : " * ");
        const std::string cast = "(" + tn(type(w[0])->kind == TypeKind::Vector ? type(w[0])->component : w[0]) + ")";
        cw(w[1], w[0], {w[2], w[3]}, [&](auto& c) { return cast + "((uint32_t)" + c[0] + op + "(uint32_t)" + c[1] + ")"; });
        return true;
    }
    case OpUDiv: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[1] + " == 0u ? 0u : (uint32_t)" + c[0] + " / (uint32_t)" + c[1] + ")"; }); return true;
    case OpUMod: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[1] + " == 0u ? 0u : (uint32_t)" + c[0] + " % (uint32_t)" + c[1] + ")"; }); return true;
    case OpSDiv: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[1] + " == 0 ? 0 : (int32_t)" + c[0] + " / (int32_t)" + c[1] + ")"; }); return true;
    case OpSRem: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[1] + " == 0 ? 0 : (int32_t)" + c[0] + " % (int32_t)" + c[1] + ")"; }); return true;
    case OpSMod:
        cw(w[1], w[0], {w[2], w[3]}, [](auto& c) {
            return "(" + c[1] + " == 0 ? 0 : ((((int32_t)" + c[0] + " % (int32_t)" + c[1] + ") + (int32_t)" + c[1] + ") % (int32_t)" + c[1] + "))";
        });
        return true;
    case OpShiftRightLogical: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((uint32_t)" + c[0] + " >> (" + c[1] + " & 31))"; }); return true;
    case OpShiftRightArithmetic: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((int32_t)" + c[0] + " >> (" + c[1] + " & 31))"; }); return true;
    case OpShiftLeftLogical: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((uint32_t)" + c[0] + " << (" + c[1] + " & 31))"; }); return true;
    case OpBitwiseOr: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " | " + c[1] + ")"; }); return true;
    case OpBitwiseXor: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " ^ " + c[1] + ")"; }); return true;
    case OpBitwiseAnd: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " & " + c[1] + ")"; }); return true;
    case OpNot: cw(w[1], w[0], {w[2]}, [](auto& c) { return "(~" + c[0] + ")"; }); return true;
    // ---- conversions ----
    case OpConvertFToS: cw(w[1], w[0], {w[2]}, [](auto& c) { return "__float2int_rz(" + c[0] + ")"; }); return true;
    case OpConvertFToU: cw(w[1], w[0], {w[2]}, [](auto& c) { return "__float2uint_rz(" + c[0] + ")"; }); return true;
    case OpConvertSToF: cw(w[1], w[0], {w[2]}, [](auto& c) { return "__int2float_rn(" + c[0] + ")"; }); return true;
    case OpConvertUToF: cw(w[1], w[0], {w[2]}, [](auto& c) { return "__uint2float_rn(" + c[0] + ")"; }); return true;
    case OpUConvert: case OpSConvert: case OpFConvert:
        cw(w[1], w[0], {w[2]}, [](auto& c) { return c[0]; });
        return true;
    case OpBitcast: {
        const Type* rt = type(w[0]);
        const uint32_t rel = rt->kind == TypeKind::Vector ? rt->component : w[0];
        const Type* st = type(type_of(w[2]));
        const uint32_t sel = st->kind == TypeKind::Vector ? st->component : type_of(w[2]);
        const bool to_f = is_float_scalar(rel), from_f = is_float_scalar(sel);
        const std::string relt = tn(rel);
        cw(w[1], w[0], {w[2]}, [&](auto& c) {
            if (to_f && !from_f) return "__uint_as_float((uint32_t)" + c[0] + ")";
            if (!to_f && from_f) return "(" + relt + ")__float_as_uint(" + c[0] + ")";
            return "(" + relt + ")" + c[0];
        });
        return true;
    }
    // ---- vector/matrix ----
    case OpVectorTimesScalar: body_ << "  " << R(w[1]) << " = cpv_vec_times_scalar(" << value(w[2]) << ", " << value(w[3]) << ");\n"; return true;
    case OpMatrixTimesScalar: body_ << "  " << R(w[1]) << " = cpv_mat_times_scalar(" << value(w[2]) << ", " << value(w[3]) << ");\n"; return true;
    case OpMatrixTimesVector: body_ << "  " << R(w[1]) << " = cpv_mat_times_vec(" << value(w[2]) << ", " << value(w[3]) << ");\n"; return true;
    case OpDot: body_ << "  " << R(w[1]) << " = cpv_dot(" << value(w[2]) << ", " << value(w[3]) << ");\n"; return true;
    case OpVectorTimesMatrix:
    case OpMatrixTimesMatrix:
    case OpTranspose:
        return fail("matrix operation " + std::to_string(ins.opcode) + " is not supported");
    // ---- comparisons / logic ----
    case OpFOrdEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " == " + c[1] + ")"; }); return true;
    case OpFUnordEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "!(" + c[0] + " < " + c[1] + " || " + c[0] + " > " + c[1] + ")"; }); return true;
    case OpFOrdNotEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " < " + c[1] + " || " + c[0] + " > " + c[1] + ")"; }); return true;
    case OpFUnordNotEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " != " + c[1] + ")"; }); return true;
    case OpFOrdLessThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " < " + c[1] + ")"; }); return true;
    case OpFUnordLessThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "!(" + c[0] + " >= " + c[1] + ")"; }); return true;
    case OpFOrdGreaterThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " > " + c[1] + ")"; }); return true;
    case OpFUnordGreaterThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "!(" + c[0] + " <= " + c[1] + ")"; }); return true;
    case OpFOrdLessThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " <= " + c[1] + ")"; }); return true;
    case OpFUnordLessThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "!(" + c[0] + " > " + c[1] + ")"; }); return true;
    case OpFOrdGreaterThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " >= " + c[1] + ")"; }); return true;
    case OpFUnordGreaterThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "!(" + c[0] + " < " + c[1] + ")"; }); return true;
    case OpIEqual: case OpLogicalEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " == " + c[1] + ")"; }); return true;
    case OpINotEqual: case OpLogicalNotEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " != " + c[1] + ")"; }); return true;
    case OpUGreaterThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((uint32_t)" + c[0] + " > (uint32_t)" + c[1] + ")"; }); return true;
    case OpSGreaterThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((int32_t)" + c[0] + " > (int32_t)" + c[1] + ")"; }); return true;
    case OpUGreaterThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((uint32_t)" + c[0] + " >= (uint32_t)" + c[1] + ")"; }); return true;
    case OpSGreaterThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((int32_t)" + c[0] + " >= (int32_t)" + c[1] + ")"; }); return true;
    case OpULessThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((uint32_t)" + c[0] + " < (uint32_t)" + c[1] + ")"; }); return true;
    case OpSLessThan: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((int32_t)" + c[0] + " < (int32_t)" + c[1] + ")"; }); return true;
    case OpULessThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((uint32_t)" + c[0] + " <= (uint32_t)" + c[1] + ")"; }); return true;
    case OpSLessThanEqual: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "((int32_t)" + c[0] + " <= (int32_t)" + c[1] + ")"; }); return true;
    case OpLogicalOr: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " || " + c[1] + ")"; }); return true;
    case OpLogicalAnd: cw(w[1], w[0], {w[2], w[3]}, [](auto& c) { return "(" + c[0] + " && " + c[1] + ")"; }); return true;
    case OpLogicalNot: cw(w[1], w[0], {w[2]}, [](auto& c) { return "(!" + c[0] + ")"; }); return true;
    case OpIsNan: cw(w[1], w[0], {w[2]}, [](auto& c) { return "isnan(" + c[0] + ")"; }); return true;
    case OpIsInf: cw(w[1], w[0], {w[2]}, [](auto& c) { return "isinf(" + c[0] + ")"; }); return true;
    case OpSelect: {
        const Type* ct = type(type_of(w[2]));
        if (ct && ct->kind == TypeKind::Vector) cw(w[1], w[0], {w[2], w[3], w[4]}, [](auto& c) { return "(" + c[0] + " ? " + c[1] + " : " + c[2] + ")"; });
        else body_ << "  " << R(w[1]) << " = " << value(w[2]) << " ? " << value(w[3]) << " : " << value(w[4]) << ";\n";
        return true;
    }
    case OpAny:
    case OpAll: {
        const Type* t = type(type_of(w[2]));
        std::string e = ins.opcode == OpAny ? "false" : "true";
        for (uint32_t i = 0; i < t->count; i++) e = "(" + e + (ins.opcode == OpAny ? " || " : " && ") + comp(w[2], i) + ")";
        body_ << "  " << R(w[1]) << " = " << e << ";\n";
        return true;
    }
    // ---- extended instructions (GLSL.std.450) ----
    case OpExtInst: {
        auto imp = m_.ext_imports.find(w[2]);
        if (imp == m_.ext_imports.end() || imp->second != "GLSL.std.450") return fail("unsupported extended instruction set");
        const uint32_t inst = w[3];
        std::vector<uint32_t> a(w.begin() + 4, w.end());
        auto call = [&](const std::string& fn) {
            std::string s = "  " + R(w[1]) + " = " + fn + "(";
            for (size_t i = 0; i < a.size(); i++) s += (i ? ", " : "") + value(a[i]);
            body_ << s << ");\n";
        };
        switch (inst) {
        case 4: cw(w[1], w[0], a, [](auto& c) { return "fabsf(" + c[0] + ")"; }); return true;
        case 5: cw(w[1], w[0], a, [](auto& c) { return "abs(" + c[0] + ")"; }); return true;
        case 6: cw(w[1], w[0], a, [](auto& c) { return "(" + c[0] + " > 0.0f ? 1.0f : (" + c[0] + " < 0.0f ? -1.0f : 0.0f))"; }); return true;
        case 7: cw(w[1], w[0], a, [](auto& c) { return "((0 < (" + c[0] + ")) - ((" + c[0] + ") < 0))"; }); return true;  // SSign
        case 8: cw(w[1], w[0], a, [](auto& c) { return "floorf(" + c[0] + ")"; }); return true;
        case 9: cw(w[1], w[0], a, [](auto& c) { return "ceilf(" + c[0] + ")"; }); return true;
        case 10: cw(w[1], w[0], a, [](auto& c) { return "__fsub_rn(" + c[0] + ", floorf(" + c[0] + "))"; }); return true;
        case 13: cw(w[1], w[0], a, [](auto& c) { return "sinf(" + c[0] + ")"; }); return true;
        case 14: cw(w[1], w[0], a, [](auto& c) { return "cosf(" + c[0] + ")"; }); return true;
        case 15: cw(w[1], w[0], a, [](auto& c) { return "tanf(" + c[0] + ")"; }); return true;
        case 26: call("cpv_glsl_pow"); return true;
        case 27: cw(w[1], w[0], a, [](auto& c) { return "expf(" + c[0] + ")"; }); return true;
        case 28: cw(w[1], w[0], a, [](auto& c) { return "logf(" + c[0] + ")"; }); return true;
        case 29: cw(w[1], w[0], a, [](auto& c) { return "exp2f(" + c[0] + ")"; }); return true;
        case 30: cw(w[1], w[0], a, [](auto& c) { return "log2f(" + c[0] + ")"; }); return true;
        case 31: cw(w[1], w[0], a, [](auto& c) { return "__fsqrt_rn(" + c[0] + ")"; }); return true;
        case 32: cw(w[1], w[0], a, [](auto& c) { return "__fdiv_rn(1.0f, __fsqrt_rn(" + c[0] + "))"; }); return true;
        case 37: call("cpv_glsl_fmin"); return true;
        case 40: call("cpv_glsl_fmax"); return true;
        case 38: case 39: cw(w[1], w[0], a, [](auto& c) { return "((" + c[1] + " < " + c[0] + ") ? " + c[1] + " : " + c[0] + ")"; }); return true;
        case 41: case 42: cw(w[1], w[0], a, [](auto& c) { return "((" + c[0] + " < " + c[1] + ") ? " + c[1] + " : " + c[0] + ")"; }); return true;
        case 43: call("cpv_glsl_fclamp"); return true;
        case 44: case 45:
            cw(w[1], w[0], a, [](auto& c) { return "((" + c[0] + " < " + c[1] + ") ? " + c[1] + " : ((" + c[2] + " < " + c[0] + ") ? " + c[2] + " : " + c[0] + "))"; });
            return true;
        case 46: call("cpv_glsl_fmix"); return true;
        case 48: cw(w[1], w[0], a, [](auto& c) { return "((" + c[1] + " < " + c[0] + ") ? 0.0f : 1.0f)"; }); return true;
        case 66: {
            const Type* t = type(type_of(a[0]));
            if (t && t->kind == TypeKind::Vector) body_ << "  " << R(w[1]) << " = __fsqrt_rn(cpv_dot(" << value(a[0]) << ", " << value(a[0]) << "));\n";
            else body_ << "  " << R(w[1]) << " = fabsf(" << value(a[0]) << ");\n";
            return true;
        }
        case 69: call("cpv_normalize"); return true;
        case 71: call("cpv_glsl_reflect"); return true;
        case 73: cw(w[1], w[0], a, [](auto& c) { return "cpv_find_ilsb((uint32_t)(" + c[0] + "))"; }); return true;
        case 74: cw(w[1], w[0], a, [](auto& c) { return "cpv_find_smsb((int32_t)(" + c[0] + "))"; }); return true;
        case 75: cw(w[1], w[0], a, [](auto& c) { return "cpv_find_umsb((uint32_t)(" + c[0] + "))"; }); return true;
        case 79: call("cpv_glsl_nmin"); return true;
        case 80: call("cpv_glsl_nmax"); return true;
        case 81: call("cpv_glsl_nclamp"); return true;
        default:
            return fail("unsupported GLSL.std.450 instruction " + std::to_string(inst));
        }
    }
    // ---- images ----
    case OpSampledImage: {
        // a sampled image from an image and a sampler in separate bindings
        // (LLVMRuntime/SPIRVCompiler.cpp:2459-2466 passes both descriptors);
        // each pair is a texture slot the ICD fills from both
        auto im = images_.find(w[2]);
        auto sm = samplers_.find(w[3]);
        if (im == images_.end() || sm == samplers_.end()) return fail("OpSampledImage of an unknown image or sampler");
        const Type* it = type(im->second.type);
        if (it && it->sampled == 2) return fail("sampling a storage image");
        const uint32_t slot = slot_for_pair(im->second, sm->second);
        if (slot >= 4) return fail("more than 4 sampled images");
        handles_[w[1]] = slot;
        return true;
    }
    case OpImageRead: {
        // imageLoad (CPVulkan/GlslFunctions.cpp:740-744): the reference's
        // ImageFetch — level 0 of the view, zeros outside it; no image
        // operands (LLVMRuntime/SPIRVCompiler.cpp:1655-1674)
        if (w.size() > 4) return fail("image operands on OpImageRead");
        auto im = images_.find(w[2]);
        if (im == images_.end()) return fail("reading an unknown image");
        const Type* it = type(im->second.type);
        // the draw path's images are 8-bit RGBA: Rgba8 (4) or Unknown (0)
        if (!it || it->sampled != 2 || (it->image_format != 4 && it->image_format != 0)) return fail("only rgba8 storage images can be read");
        const uint32_t slot = slot_for(im->second.set, im->second.binding, true);
        if (slot >= 4) return fail("more than 4 sampled images");
        samples_++;
        body_ << "  " << R(w[1]) << " = cpv_fetch(P.tex[" << slot << "], (int32_t)" << comp(w[3], 0) << ", (int32_t)" << comp(w[3], 1) << ");\n";
        return true;
    }
    case OpImageWrite:
        // fragments run concurrently here, and Vulkan leaves the order of
        // their image stores undefined: no image writes from the draw path
        return fail("image writes (imageStore) are not supported on the draw path");
    case OpImage: {
        // the image of a sampled image (LLVMRuntime/SPIRVCompiler.cpp:2480-2519)
        auto h = handles_.find(w[2]);
        if (h == handles_.end()) return fail("OpImage of an unknown sampled image");
        handles_[w[1]] = h->second;
        return true;
    }
    case OpImageFetch: {
        // texelFetch (CPVulkan/GlslFunctions.cpp:674-742): level 0 whatever
        // the Lod operand, integer texel coordinates, zero outside the level
        uint32_t slot = 0;
        auto h = handles_.find(w[2]);
        auto im = images_.find(w[2]);
        if (h != handles_.end()) {
            slot = h->second;
        } else if (im != images_.end()) {
            slot = slot_for(im->second.set, im->second.binding, true);
            if (slot >= 4) return fail("more than 4 sampled images");
        } else {
            return fail("fetching from an unknown image");
        }
        samples_++;
        body_ << "  " << R(w[1]) << " = cpv_fetch(P.tex[" << slot << "], (int32_t)" << comp(w[3], 0) << ", (int32_t)" << comp(w[3], 1) << ");\n";
        return true;
    }
    case OpBitCount:
        cw(w[1], w[0], {w[2]}, [](auto& c) { return "__popc((uint32_t)" + c[0] + ")"; });
        return true;
    case OpCopyMemory: {
        // a copy of the source object into the target (:2008-2019)
        auto dst = ptrs_.find(w[0]);
        auto src = ptrs_.find(w[1]);
        if (dst == ptrs_.end() || src == ptrs_.end()) return fail("copy through an unknown pointer");
        if (dst->second.kind != PtrInfo::Lvalue) return fail("copy to read-only memory");
        const PtrInfo& p = src->second;
        if (p.kind == PtrInfo::Lvalue) body_ << "  " << dst->second.lvalue << " = " << p.lvalue << ";\n";
        else if (p.kind == PtrInfo::Explicit)
            body_ << "  " << dst->second.lvalue << " = " << loader(p.type) << "(" << p.base << ", " << p.bytes << ", " << p.offset << ", " << p.mstride << "u);\n";
        else return fail("copy of an image handle");
        return true;
    }
    case OpImageSampleImplicitLod:
    case OpImageSampleExplicitLod: {
        auto h = handles_.find(w[2]);
        if (h == handles_.end()) return fail("sampling through an unknown image");
        std::string lod = "0.0f";
        if (ins.opcode == OpImageSampleExplicitLod) {
            if (w.size() < 6 || !(w[4] & 0x2u)) return fail("explicit-LOD sampling without a Lod operand");
            lod = value(w[5]);
        }
        samples_++;
        if (ins.opcode == OpImageSampleImplicitLod && spec_lod_) {
            // λ from the coordinates of the quad's neighbours at this
            // instruction (one site per instruction)
            body_ << "  " << R(w[1]) << " = cpv_sample_quad(P.tex[" << h->second << "], " << comp(w[3], 0) << ", " << comp(w[3], 1) << ", cpv_lod, "
                  << lod_sites_ << ");\n";
            lod_sites_++;
            return true;
        }
        body_ << "  " << R(w[1]) << " = cpv_sample(P.tex[" << h->second << "], " << comp(w[3], 0) << ", " << comp(w[3], 1) << ", " << lod << ");\n";
        return true;
    }
    // ---- control flow ----
    case OpBranch:
        edge_copies();
        body_ << "  goto L" << w[0] << ";\n";
        return true;
    case OpBranchConditional:
        edge_copies();
        body_ << "  if (" << value(w[0]) << ") goto L" << w[1] << "; else goto L" << w[2] << ";\n";
        return true;
    case OpSwitch: {
        edge_copies();
        body_ << "  switch (" << value(w[0]) << ") {\n";
        for (size_t k = 2; k + 1 < w.size(); k += 2) body_ << "  case " << w[k] << "u: goto L" << w[k + 1] << ";\n";
        body_ << "  default: goto L" << w[1] << ";\n  }\n";
        return true;
    }
    case OpReturn:
        body_ << (callee_ ? "  return;\n" : "  goto cpv_epilogue;\n");
        return true;
    case OpKill:
        if (model_ != 4) return fail("OpKill outside a fragment shader");
        has_kill_ = true;
        // a discard inside a called function ends the whole invocation: the
        // callers return too (cpv_killed, checked after every call)
        if (callee_) body_ << "  cpv_killed = true;\n  return" << callee_default_return() << ";\n";
        else body_ << "  return true;\n";
        return true;
    case OpUnreachable:
        if (callee_) body_ << "  return" << callee_default_return() << ";\n";
        else body_ << "  goto cpv_epilogue;\n";
        return true;
    case OpReturnValue:
        if (!callee_) return fail("OpReturnValue in the entry point");
        body_ << "  return " << value(w[0]) << ";\n";
        return true;
    case OpFunctionCall: {
        // (LLVMRuntime/SPIRVCompiler.cpp translates every function; here each
        // is a lambda of the stage function, called with its arguments: a
        // pointer argument passes the variable it points at by reference)
        std::string call = "f" + std::to_string(w[2]) + "(";
        for (size_t k = 3; k < w.size(); k++) {
            auto pit = ptrs_.find(w[k]);
            if (pit != ptrs_.end()) {
                if (pit->second.kind != PtrInfo::Lvalue) return fail("a function argument points at a uniform, image or input");
                call += (k > 3 ? ", " : "") + pit->second.lvalue;
            } else {
                call += (k > 3 ? ", " : "") + value(w[k]);
            }
        }
        call += ")";
        const Type* rt = type(w[0]);
        if (rt && rt->kind != TypeKind::Void) body_ << "  " << R(w[1]) << " = " << call << ";\n";
        else body_ << "  " << call << ";\n";
        if (model_ == 4 && has_kill_) {
            if (callee_) body_ << "  if (cpv_killed) return" << callee_default_return() << ";\n";
            else body_ << "  if (cpv_killed) return true;\n";
        }
        return true;
    }
    default:
        return fail("unsupported SPIR-V opcode " + std::to_string(ins.opcode));
    }
}

std::string Translator::callee_default_return() {
    const Type* rt = callee_ ? type(callee_->result_type) : nullptr;
    if (!rt || rt->kind == TypeKind::Void) return "";
    return " " + tn(callee_->result_type) + "{}";
}

// Functions reachable from `fid`, callees before their callers; recursion
// (which SPIR-V shaders may not use) is rejected.
bool Translator::order_callees(uint32_t fid, std::vector<uint32_t>& order, std::set<uint32_t>& seen, std::set<uint32_t>& stack) {
    auto fit = m_.functions.find(fid);
    if (fit == m_.functions.end()) return fail("call of an unknown function");
    stack.insert(fid);
    for (const Block& b : fit->second.blocks)
        for (const Instruction& ins : b.body) {
            if (ins.opcode != OpFunctionCall || ins.words.size() < 3) continue;
            const uint32_t callee = ins.words[2];
            if (stack.count(callee)) return fail("recursive function call");
            if (seen.count(callee)) continue;
            seen.insert(callee);
            if (!order_callees(callee, order, seen, stack)) return false;
            order.push_back(callee);
        }
    stack.erase(fid);
    return true;
}

// A function other than the entry point as a lambda of the stage function:
// value parameters by value, pointer parameters (to Function or Private
// variables) as references to the caller's variable.
bool Translator::emit_callee(const Function& f) {
    std::ostringstream decls, pro, body;
    std::swap(decls, decls_);
    std::swap(pro, pro_);
    std::swap(body, body_);
    callee_ = &f;
    std::string params;
    bool ok = true;
    for (size_t i = 0; i < f.params.size() && ok; i++) {
        const uint32_t pid = f.params[i];
        const Type* t = type(f.param_types[i]);
        if (!t) {
            ok = fail("bad function parameter type");
            break;
        }
        if (i) params += ", ";
        if (t->kind == TypeKind::Pointer) {
            if (t->storage != SCFunction && t->storage != SCPrivate) {
                ok = fail("a function parameter points at a uniform, image or input");
                break;
            }
            PtrInfo info;
            info.kind = PtrInfo::Lvalue;
            info.lvalue = "v" + std::to_string(pid);
            info.type = t->component;
            ptrs_[pid] = info;
            params += tn(t->component) + "& v" + std::to_string(pid);
        } else {
            if (t->kind == TypeKind::SampledImage || t->kind == TypeKind::Image || t->kind == TypeKind::Sampler) {
                ok = fail("an image or sampler function parameter");
                break;
            }
            value_type_[pid] = f.param_types[i];
            params += tn(f.param_types[i]) + " r" + std::to_string(pid);
        }
    }
    if (ok) ok = emit_function(f);
    const Type* rt = type(f.result_type);
    const bool has_value = rt && rt->kind != TypeKind::Void;
    std::swap(decls, decls_);
    std::swap(pro, pro_);
    std::swap(body, body_);
    if (ok) {
        funcs_ << "  auto f" << f.id << " = [&](" << params << ") -> " << (has_value ? tn(f.result_type) : std::string("void")) << " {\n"
               << decls.str() << pro.str() << body.str();
        if (has_value) funcs_ << "  return " << tn(f.result_type) << "{};\n";
        funcs_ << "  };\n";
    }
    callee_ = nullptr;
    return ok && err_.empty();
}

bool Translator::run(const std::string& entry_name, StageResult& out, std::string& error) {
    const EntryPoint* ep = m_.find_entry(model_, entry_name);
    if (!ep) {
        error = "entry point '" + entry_name + "' not found for this stage";
        return false;
    }
    auto fit = m_.functions.find(ep->function);
    if (fit == m_.functions.end()) {
        error = "entry function missing";
        return false;
    }
    out.origin_upper_left = true;
    auto modes = m_.exec_modes.find(ep->function);
    if (modes != m_.exec_modes.end()) {
        for (uint32_t md : modes->second) {
            if (md == 8) out.origin_upper_left = false;
            if (md == 12) {
                error = "DepthReplacing is not supported";
                return false;
            }
        }
    }
    std::vector<uint32_t> callees;
    std::set<uint32_t> seen, stack;
    bool ok = emit_globals(*ep, out) && order_callees(ep->function, callees, seen, stack);
    for (size_t i = 0; ok && i < callees.size(); i++) ok = emit_callee(m_.functions.at(callees[i]));
    if (!ok || !emit_function(fit->second)) {
        error = err_.empty() ? "translation failed" : err_;
        return false;
    }
    out.has_kill = has_kill_;
    out.samples = samples_;
    out.lod_sites = lod_sites_;
    out.instructions = instructions_;
    out.outputs = out_outputs_;
    const std::string ns = model_ == 0 ? "cpv_vs_ns" : "cpv_fs_ns";
    std::ostringstream s;
    s << "namespace " << ns << " {\n" << types_.str() << loaders_.str() << "}\n";
    if (model_ == 0) {
        s << "__device__ __forceinline__ void cpv_vs_run(const CpvDrawParams& P, uint32_t cpv_vertex_index, uint32_t cpv_instance_index, "
             "float* cpv_pos, float* cpv_var, float* cpv_point_size = nullptr) {\n";
        s << "  using namespace " << ns << ";\n";
        s << "  for (int i = 0; i < CPV_NV; i++) cpv_var[i] = 0.0f;\n";
        s << "  cpv_pos[0] = cpv_pos[1] = cpv_pos[2] = 0.0f; cpv_pos[3] = 1.0f;\n";
    } else {
        s << "__device__ __forceinline__ bool cpv_fs_run(const CpvDrawParams& P, const float* cpv_in, const float* cpv_frag_coord, "
             "bool cpv_front, float* cpv_colour" << (spec_lod_ ? ", CpvQuadLod* cpv_lod = nullptr" : "") << ") {\n";
        s << "  using namespace " << ns << ";\n  (void)cpv_in; (void)cpv_frag_coord; (void)cpv_front;\n";
        if (spec_lod_) s << "  (void)cpv_lod;\n";
        s << "  cpv_colour[0] = cpv_colour[1] = cpv_colour[2] = 0.0f; cpv_colour[3] = 1.0f;\n";
    }
    if (!callees.empty() && model_ == 4) s << "  bool cpv_killed = false;\n  (void)cpv_killed;\n";
    s << decls_.str() << pro_.str() << funcs_.str() << body_.str() << " cpv_epilogue:;\n" << epi_.str();
    if (model_ != 0) s << "  return false;\n";
    s << "}\n";
    out.code = s.str();
    return true;
}

}  // namespace

bool translate_stage(const Module& m, uint32_t model, const std::string& entry, const std::vector<SpecConstant>& spec,
                     const std::vector<VertexBinding>& bindings, const std::vector<VertexAttribute>& attributes,
                     std::vector<ResourceSlot>& slots, StageResult& out, std::string& error, bool spec_lod) {
    Translator t(m, model, spec, bindings, attributes, slots, spec_lod);
    return t.run(entry, out, error);
}

}  // namespace cpv::spirv
