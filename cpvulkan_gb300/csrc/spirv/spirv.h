// spirv.h — a small SPIR-V 1.x module reader and the SPIR-V → CUDA C++
// translator used at vkCreateGraphicsPipelines.
//
// Replaces the reference's vendored SPIRV-LLVM-Translator reader
// (SPIRVParser/) and its SPIR-V → LLVM IR builder (LLVMRuntime/SPIRVCompiler.cpp):
// instead of LLVM IR for an ORC JIT, each stage becomes a CUDA device
// function that NVRTC compiles together with the raster kernels.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace cpv::spirv {

struct Instruction {
    uint16_t opcode = 0;
    std::vector<uint32_t> words;  // operands (without the leading opcode word)
};

enum class TypeKind { Void, Bool, Int, Float, Vector, Matrix, Array, RuntimeArray, Struct, Pointer, Function, Image, Sampler, SampledImage, Unknown };

struct Type {
    TypeKind kind = TypeKind::Unknown;
    uint32_t width = 0;       // int/float
    bool is_signed = false;   // int
    uint32_t component = 0;   // vector/matrix/array element type, pointer pointee, sampled-image image type
    uint32_t count = 0;       // vector/matrix/array length
    uint32_t storage = 0;     // pointer storage class
    std::vector<uint32_t> members;  // struct members, function param types
    uint32_t result = 0;            // function return type
    uint32_t dim = 0, sampled = 0, image_format = 0;  // image: Dim, Sampled (1 sampled, 2 storage), ImageFormat
};

struct Constant {
    uint32_t type = 0;
    std::vector<uint32_t> words;       // scalar literal words
    std::vector<uint32_t> constituents;// composite
    bool composite = false;
    bool null = false;
    bool spec = false;
    uint32_t spec_id = 0xFFFFFFFFu;
    uint32_t spec_op = 0;              // OpSpecConstantOp: the operation (operands in constituents)
};

struct Variable {
    uint32_t id = 0;
    uint32_t type = 0;  // pointer type
    uint32_t storage = 0;
    uint32_t init = 0;
};

struct Block {
    uint32_t label = 0;
    std::vector<Instruction> body;
};

struct Function {
    uint32_t id = 0;
    uint32_t result_type = 0;
    uint32_t type = 0;
    std::vector<uint32_t> params;
    std::vector<uint32_t> param_types;
    std::vector<Block> blocks;
};

struct EntryPoint {
    uint32_t model = 0;
    uint32_t function = 0;
    std::string name;
    std::vector<uint32_t> interface;
};

struct Decoration {
    uint32_t kind = 0;
    std::vector<uint32_t> literals;
};

struct Module {
    uint32_t version = 0;
    uint32_t bound = 0;
    std::map<uint32_t, Type> types;
    std::map<uint32_t, Constant> constants;
    std::vector<Variable> globals;  // declaration order
    std::map<uint32_t, Function> functions;
    std::vector<EntryPoint> entries;
    std::map<uint32_t, std::vector<uint32_t>> exec_modes;  // function → modes
    std::map<uint32_t, std::vector<Decoration>> decorations;
    std::map<std::pair<uint32_t, uint32_t>, std::vector<Decoration>> member_decorations;
    std::map<uint32_t, std::string> ext_imports;
    std::map<uint32_t, std::string> names;
    std::map<uint32_t, uint32_t> undefs;  // id → type

    bool has_decoration(uint32_t id, uint32_t kind) const;
    bool decoration(uint32_t id, uint32_t kind, uint32_t& value) const;
    bool member_decoration(uint32_t st, uint32_t member, uint32_t kind, uint32_t& value) const;
    const EntryPoint* find_entry(uint32_t model, const std::string& name) const;
};

// Parses a SPIR-V binary. Returns false and sets error on malformed input.
bool parse(const uint32_t* words, size_t word_count, Module& out, std::string& error);

// Pipeline-level facts the translator needs about the other stage and the
// fixed-function state.
struct VertexAttribute {
    uint32_t location = 0, binding = 0, format = 0, offset = 0;
};
struct VertexBinding {
    uint32_t binding = 0, stride = 0, input_rate = 0;
};

// Descriptor slots: every (set, binding) a pipeline's shaders use is given a
// dense slot in CpvDrawParams (ubo[] for uniform buffers, tex[] for combined
// image samplers, storage images read by OpImageRead, and each (sampled
// image, sampler) pair an OpSampledImage joins), shared by both stages.
struct ResourceSlot {
    uint32_t set = 0, binding = 0;
    bool is_texture = false;
    uint32_t slot = 0;
    // a texture joined from a sampled image and a sampler in another binding
    // (OpSampledImage): the sampler's (set, binding)
    bool separate = false;
    uint32_t sampler_set = 0, sampler_binding = 0;
};

struct SpecConstant {
    uint32_t id = 0;
    std::vector<uint8_t> bytes;
};

struct StageResult {
    std::string code;          // CUDA C++ (device functions)
    uint32_t num_floats = 0;   // VS: output floats; FS: input floats
    std::vector<int> interp;   // FS: per input float, 0 perspective / 1 linear / 2 flat
    bool origin_upper_left = true;
    bool has_kill = false;
    uint32_t samples = 0;      // image sampling instructions emitted
    uint32_t lod_sites = 0;    // FS with spec_lod: implicit-LOD sampling instructions (quad-derivative sites)
    uint32_t instructions = 0; // SPIR-V instructions of the entry function
    bool reads_frag_coord = false;    // FS: FragCoord is an input
    bool reads_front_facing = false;  // FS: FrontFacing is an input
    uint32_t outputs = 0;             // FS: bit L set when an output is declared at location L (< 8)
};

// Translates the entry point of `m` for `model` (0 vertex, 4 fragment) into a
// device function named cpv_vs_run / cpv_fs_run. Resource slots are appended
// to `slots` as new (set, binding) pairs are met. With spec_lod, a fragment
// shader's implicit-LOD sampling takes λ from quad derivatives of its
// coordinates (cpv_sample_quad) instead of the reference's λ = 0, and
// cpv_fs_run takes the quad's context as a last argument.
bool translate_stage(const Module& m, uint32_t model, const std::string& entry, const std::vector<SpecConstant>& spec,
                     const std::vector<VertexBinding>& bindings, const std::vector<VertexAttribute>& attributes,
                     std::vector<ResourceSlot>& slots, StageResult& out, std::string& error, bool spec_lod = false);

}  // namespace cpv::spirv
