/*
 * kz_spirv.cpp - SPIR-V decoding and text dump (see kz_spirv.h).
 *
 * Reference counterpart: spirv-parser (generated decoder, spirv-parser/src/generated_parser.rs) and its
 * dump format checked by spirv-parser/src/lib.rs:45-216.  Written here from the SPIR-V specification's
 * instruction grammar for the opcodes graphics shaders use; unknown opcodes decode generically.
 */
#include "kz_spirv.h"

#include <cstdio>
#include <cstring>
#include <unordered_map>

namespace kz {
namespace spv {

bool bytes_to_words(const uint8_t* b, size_t n, std::vector<uint32_t>& w) {
  if (n % 4) return false;
  w.resize(n / 4);
  for (size_t i = 0; i < n / 4; i++)
    w[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) | ((uint32_t)b[4 * i + 2] << 16) |
           ((uint32_t)b[4 * i + 3] << 24);
  return true;
}

std::string decode(const uint32_t* words, size_t count, Module& out) {
  if (count < 5) return "module shorter than the SPIR-V header";
  if (words[0] != kMagic) return "bad SPIR-V magic number";
  out.version = words[1];
  out.generator = words[2];
  out.bound = words[3];
  out.schema = words[4];
  out.insns.clear();
  size_t i = 5;
  while (i < count) {
    uint32_t w = words[i];
    uint32_t wc = w >> 16;
    if (wc == 0) return "instruction with zero word count";
    if (i + wc > count) return "instruction runs past the end of the module";
    Insn in;
    in.opcode = (uint16_t)(w & 0xFFFFu);
    in.offset = (uint32_t)(i * 4);
    in.ops.assign(words + i + 1, words + i + wc);
    out.insns.push_back(std::move(in));
    i += wc;
  }
  return "";
}

std::string read_string(const std::vector<uint32_t>& ops, size_t& i) {
  std::string s;
  while (i < ops.size()) {
    uint32_t w = ops[i++];
    bool end = false;
    for (int k = 0; k < 4; k++) {
      char c = (char)((w >> (8 * k)) & 0xFFu);
      if (c == 0) {
        end = true;
        break;
      }
      s.push_back(c);
    }
    if (end) break;
  }
  return s;
}

namespace {

struct OpInfo {
  uint16_t op;
  const char* name;
  const char* grammar;
};

/* grammar letters: t result type, r result id, i id, I ids to the end, l literal, L literals to the end,
 * s string, c constant literal words (hex), eX enumerant of kind X, ? the rest is optional.
 * Enumerant kinds: C capability, A addressing model, M memory model, X execution model, O execution mode,
 * S storage class, F function control, Q selection control, P loop control, G source language,
 * N memory access, Y image operands. */
const OpInfo kOps[] = {
    {OpNop, "OpNop", ""},
    {OpUndef, "OpUndef", "tr"},
    {OpSourceContinued, "OpSourceContinued", "s"},
    {OpSource, "OpSource", "eGl?is"},
    {OpSourceExtension, "OpSourceExtension", "s"},
    {OpName, "OpName", "is"},
    {OpMemberName, "OpMemberName", "ils"},
    {OpString, "OpString", "rs"},
    {OpLine, "OpLine", "ill"},
    {OpExtension, "OpExtension", "s"},
    {OpExtInstImport, "OpExtInstImport", "rs"},
    {OpExtInst, "OpExtInst", "*"},
    {OpMemoryModel, "OpMemoryModel", "eAeM"},
    {OpEntryPoint, "OpEntryPoint", "eXisI"},
    {OpExecutionMode, "OpExecutionMode", "ieOL"},
    {OpCapability, "OpCapability", "eC"},
    {OpTypeVoid, "OpTypeVoid", "r"},
    {OpTypeBool, "OpTypeBool", "r"},
    {OpTypeInt, "OpTypeInt", "rll"},
    {OpTypeFloat, "OpTypeFloat", "rl"},
    {OpTypeVector, "OpTypeVector", "ril"},
    {OpTypeMatrix, "OpTypeMatrix", "ril"},
    {OpTypeImage, "OpTypeImage", "riL"},
    {OpTypeSampler, "OpTypeSampler", "r"},
    {OpTypeSampledImage, "OpTypeSampledImage", "ri"},
    {OpTypeArray, "OpTypeArray", "rii"},
    {OpTypeRuntimeArray, "OpTypeRuntimeArray", "ri"},
    {OpTypeStruct, "OpTypeStruct", "rI"},
    {OpTypeOpaque, "OpTypeOpaque", "rs"},
    {OpTypePointer, "OpTypePointer", "reSi"},
    {OpTypeFunction, "OpTypeFunction", "riI"},
    {OpConstantTrue, "OpConstantTrue", "tr"},
    {OpConstantFalse, "OpConstantFalse", "tr"},
    {OpConstant, "OpConstant", "trc"},
    {OpConstantComposite, "OpConstantComposite", "trI"},
    {OpConstantNull, "OpConstantNull", "tr"},
    {OpSpecConstantTrue, "OpSpecConstantTrue", "tr"},
    {OpSpecConstantFalse, "OpSpecConstantFalse", "tr"},
    {OpSpecConstant, "OpSpecConstant", "trc"},
    {OpSpecConstantComposite, "OpSpecConstantComposite", "trI"},
    {OpSpecConstantOp, "OpSpecConstantOp", "*"},
    {OpFunction, "OpFunction", "treFi"},
    {OpFunctionParameter, "OpFunctionParameter", "tr"},
    {OpFunctionEnd, "OpFunctionEnd", ""},
    {OpFunctionCall, "OpFunctionCall", "triI"},
    {OpVariable, "OpVariable", "treS?i"},
    {OpImageTexelPointer, "OpImageTexelPointer", "triii"},
    {OpLoad, "OpLoad", "tri?eN"},
    {OpStore, "OpStore", "ii?eN"},
    {OpCopyMemory, "OpCopyMemory", "ii?eN"},
    {OpAccessChain, "OpAccessChain", "triI"},
    {OpInBoundsAccessChain, "OpInBoundsAccessChain", "triI"},
    {OpPtrAccessChain, "OpPtrAccessChain", "triiI"},
    {OpDecorate, "OpDecorate", "*"},
    {OpMemberDecorate, "OpMemberDecorate", "*"},
    {OpVectorExtractDynamic, "OpVectorExtractDynamic", "trii"},
    {OpVectorInsertDynamic, "OpVectorInsertDynamic", "triii"},
    {OpVectorShuffle, "OpVectorShuffle", "triiL"},
    {OpCompositeConstruct, "OpCompositeConstruct", "trI"},
    {OpCompositeExtract, "OpCompositeExtract", "triL"},
    {OpCompositeInsert, "OpCompositeInsert", "triiL"},
    {OpCopyObject, "OpCopyObject", "tri"},
    {OpTranspose, "OpTranspose", "tri"},
    {OpSampledImage, "OpSampledImage", "trii"},
    {OpImageSampleImplicitLod, "OpImageSampleImplicitLod", "trii?eYI"},
    {OpImageSampleExplicitLod, "OpImageSampleExplicitLod", "triieYI"},
    {OpConvertFToU, "OpConvertFToU", "tri"},
    {OpConvertFToS, "OpConvertFToS", "tri"},
    {OpConvertSToF, "OpConvertSToF", "tri"},
    {OpConvertUToF, "OpConvertUToF", "tri"},
    {OpUConvert, "OpUConvert", "tri"},
    {OpSConvert, "OpSConvert", "tri"},
    {OpFConvert, "OpFConvert", "tri"},
    {OpBitcast, "OpBitcast", "tri"},
    {OpSNegate, "OpSNegate", "tri"},
    {OpFNegate, "OpFNegate", "tri"},
    {OpIAdd, "OpIAdd", "trii"},
    {OpFAdd, "OpFAdd", "trii"},
    {OpISub, "OpISub", "trii"},
    {OpFSub, "OpFSub", "trii"},
    {OpIMul, "OpIMul", "trii"},
    {OpFMul, "OpFMul", "trii"},
    {OpUDiv, "OpUDiv", "trii"},
    {OpSDiv, "OpSDiv", "trii"},
    {OpFDiv, "OpFDiv", "trii"},
    {OpUMod, "OpUMod", "trii"},
    {OpSRem, "OpSRem", "trii"},
    {OpSMod, "OpSMod", "trii"},
    {OpFRem, "OpFRem", "trii"},
    {OpFMod, "OpFMod", "trii"},
    {OpVectorTimesScalar, "OpVectorTimesScalar", "trii"},
    {OpMatrixTimesScalar, "OpMatrixTimesScalar", "trii"},
    {OpVectorTimesMatrix, "OpVectorTimesMatrix", "trii"},
    {OpMatrixTimesVector, "OpMatrixTimesVector", "trii"},
    {OpMatrixTimesMatrix, "OpMatrixTimesMatrix", "trii"},
    {OpOuterProduct, "OpOuterProduct", "trii"},
    {OpDot, "OpDot", "trii"},
    {OpAny, "OpAny", "tri"},
    {OpAll, "OpAll", "tri"},
    {OpIsNan, "OpIsNan", "tri"},
    {OpIsInf, "OpIsInf", "tri"},
    {OpLogicalEqual, "OpLogicalEqual", "trii"},
    {OpLogicalNotEqual, "OpLogicalNotEqual", "trii"},
    {OpLogicalOr, "OpLogicalOr", "trii"},
    {OpLogicalAnd, "OpLogicalAnd", "trii"},
    {OpLogicalNot, "OpLogicalNot", "tri"},
    {OpSelect, "OpSelect", "triii"},
    {OpIEqual, "OpIEqual", "trii"},
    {OpINotEqual, "OpINotEqual", "trii"},
    {OpUGreaterThan, "OpUGreaterThan", "trii"},
    {OpSGreaterThan, "OpSGreaterThan", "trii"},
    {OpUGreaterThanEqual, "OpUGreaterThanEqual", "trii"},
    {OpSGreaterThanEqual, "OpSGreaterThanEqual", "trii"},
    {OpULessThan, "OpULessThan", "trii"},
    {OpSLessThan, "OpSLessThan", "trii"},
    {OpULessThanEqual, "OpULessThanEqual", "trii"},
    {OpSLessThanEqual, "OpSLessThanEqual", "trii"},
    {OpFOrdEqual, "OpFOrdEqual", "trii"},
    {OpFUnordEqual, "OpFUnordEqual", "trii"},
    {OpFOrdNotEqual, "OpFOrdNotEqual", "trii"},
    {OpFUnordNotEqual, "OpFUnordNotEqual", "trii"},
    {OpFOrdLessThan, "OpFOrdLessThan", "trii"},
    {OpFUnordLessThan, "OpFUnordLessThan", "trii"},
    {OpFOrdGreaterThan, "OpFOrdGreaterThan", "trii"},
    {OpFUnordGreaterThan, "OpFUnordGreaterThan", "trii"},
    {OpFOrdLessThanEqual, "OpFOrdLessThanEqual", "trii"},
    {OpFUnordLessThanEqual, "OpFUnordLessThanEqual", "trii"},
    {OpFOrdGreaterThanEqual, "OpFOrdGreaterThanEqual", "trii"},
    {OpFUnordGreaterThanEqual, "OpFUnordGreaterThanEqual", "trii"},
    {OpShiftRightLogical, "OpShiftRightLogical", "trii"},
    {OpShiftRightArithmetic, "OpShiftRightArithmetic", "trii"},
    {OpShiftLeftLogical, "OpShiftLeftLogical", "trii"},
    {OpBitwiseOr, "OpBitwiseOr", "trii"},
    {OpBitwiseXor, "OpBitwiseXor", "trii"},
    {OpBitwiseAnd, "OpBitwiseAnd", "trii"},
    {OpNot, "OpNot", "tri"},
    {OpDPdx, "OpDPdx", "tri"},
    {OpDPdy, "OpDPdy", "tri"},
    {OpFwidth, "OpFwidth", "tri"},
    {OpPhi, "OpPhi", "trI"},
    {OpLoopMerge, "OpLoopMerge", "iieP"},
    {OpSelectionMerge, "OpSelectionMerge", "ieQ"},
    {OpLabel, "OpLabel", "r"},
    {OpBranch, "OpBranch", "i"},
    {OpBranchConditional, "OpBranchConditional", "iiiL"},
    {OpSwitch, "OpSwitch", "*"},
    {OpKill, "OpKill", ""},
    {OpReturn, "OpReturn", ""},
    {OpReturnValue, "OpReturnValue", "i"},
    {OpUnreachable, "OpUnreachable", ""},
    {OpModuleProcessed, "OpModuleProcessed", "s"},
};

const OpInfo* find_op(uint16_t op) {
  static std::unordered_map<uint16_t, const OpInfo*> map = [] {
    std::unordered_map<uint16_t, const OpInfo*> m;
    for (const OpInfo& o : kOps) m[o.op] = &o;
    return m;
  }();
  auto it = map.find(op);
  return it == map.end() ? nullptr : it->second;
}

struct Name {
  uint32_t v;
  const char* n;
};

const Name kCapability[] = {
    {0, "Matrix"}, {1, "Shader"}, {2, "Geometry"}, {3, "Tessellation"}, {4, "Addresses"}, {5, "Linkage"},
    {6, "Kernel"}, {7, "Vector16"}, {8, "Float16Buffer"}, {9, "Float16"}, {10, "Float64"}, {11, "Int64"},
    {12, "Int64Atomics"}, {13, "ImageBasic"}, {14, "ImageReadWrite"}, {15, "ImageMipmap"}, {17, "Pipes"},
    {18, "Groups"}, {19, "DeviceEnqueue"}, {20, "LiteralSampler"}, {21, "AtomicStorage"}, {22, "Int16"},
    {23, "TessellationPointSize"}, {24, "GeometryPointSize"}, {25, "ImageGatherExtended"},
    {27, "StorageImageMultisample"}, {28, "UniformBufferArrayDynamicIndexing"},
    {29, "SampledImageArrayDynamicIndexing"}, {30, "StorageBufferArrayDynamicIndexing"},
    {31, "StorageImageArrayDynamicIndexing"}, {32, "ClipDistance"}, {33, "CullDistance"}, {34, "ImageCubeArray"},
    {35, "SampleRateShading"}, {36, "ImageRect"}, {37, "SampledRect"}, {38, "GenericPointer"}, {39, "Int8"},
    {40, "InputAttachment"}, {41, "SparseResidency"}, {42, "MinLod"}, {43, "Sampled1D"}, {44, "Image1D"},
    {45, "SampledCubeArray"}, {46, "SampledBuffer"}, {47, "ImageBuffer"}, {48, "ImageMSArray"},
    {49, "StorageImageExtendedFormats"}, {50, "ImageQuery"}, {51, "DerivativeControl"},
    {52, "InterpolationFunction"}, {53, "TransformFeedback"}, {54, "GeometryStreams"},
    {55, "StorageImageReadWithoutFormat"}, {56, "StorageImageWriteWithoutFormat"}, {57, "MultiViewport"}};
const Name kAddressing[] = {{0, "Logical"}, {1, "Physical32"}, {2, "Physical64"}};
const Name kMemoryModel[] = {{0, "Simple"}, {1, "GLSL450"}, {2, "OpenCL"}, {3, "Vulkan"}};
const Name kExecModel[] = {{0, "Vertex"},   {1, "TessellationControl"}, {2, "TessellationEvaluation"},
                           {3, "Geometry"}, {4, "Fragment"},            {5, "GLCompute"},
                           {6, "Kernel"}};
const Name kExecMode[] = {
    {0, "Invocations"}, {1, "SpacingEqual"}, {2, "SpacingFractionalEven"}, {3, "SpacingFractionalOdd"},
    {4, "VertexOrderCw"}, {5, "VertexOrderCcw"}, {6, "PixelCenterInteger"}, {7, "OriginUpperLeft"},
    {8, "OriginLowerLeft"}, {9, "EarlyFragmentTests"}, {10, "PointMode"}, {11, "Xfb"}, {12, "DepthReplacing"},
    {14, "DepthGreater"}, {15, "DepthLess"}, {16, "DepthUnchanged"}, {17, "LocalSize"}, {18, "LocalSizeHint"},
    {19, "InputPoints"}, {20, "InputLines"}, {21, "InputLinesAdjacency"}, {22, "Triangles"},
    {23, "InputTrianglesAdjacency"}, {24, "Quads"}, {25, "Isolines"}, {26, "OutputVertices"},
    {27, "OutputPoints"}, {28, "OutputLineStrip"}, {29, "OutputTriangleStrip"}, {30, "VecTypeHint"},
    {31, "ContractionOff"}};
const Name kStorage[] = {{0, "UniformConstant"}, {1, "Input"},          {2, "Uniform"},  {3, "Output"},
                         {4, "Workgroup"},       {5, "CrossWorkgroup"}, {6, "Private"},  {7, "Function"},
                         {8, "Generic"},         {9, "PushConstant"},   {10, "AtomicCounter"},
                         {11, "Image"},          {12, "StorageBuffer"}};
const Name kDecoration[] = {
    {0, "RelaxedPrecision"}, {1, "SpecId"}, {2, "Block"}, {3, "BufferBlock"}, {4, "RowMajor"}, {5, "ColMajor"},
    {6, "ArrayStride"}, {7, "MatrixStride"}, {8, "GLSLShared"}, {9, "GLSLPacked"}, {10, "CPacked"},
    {11, "BuiltIn"}, {13, "NoPerspective"}, {14, "Flat"}, {15, "Patch"}, {16, "Centroid"}, {17, "Sample"},
    {18, "Invariant"}, {19, "Restrict"}, {20, "Aliased"}, {21, "Volatile"}, {22, "Constant"}, {23, "Coherent"},
    {24, "NonWritable"}, {25, "NonReadable"}, {26, "Uniform"}, {28, "SaturatedConversion"}, {29, "Stream"},
    {30, "Location"}, {31, "Component"}, {32, "Index"}, {33, "Binding"}, {34, "DescriptorSet"}, {35, "Offset"},
    {36, "XfbBuffer"}, {37, "XfbStride"}, {38, "FuncParamAttr"}, {39, "FPRoundingMode"},
    {40, "FPFastMathMode"}, {41, "LinkageAttributes"}, {42, "NoContraction"}, {43, "InputAttachmentIndex"},
    {44, "Alignment"}};
const Name kBuiltIn[] = {
    {0, "Position"}, {1, "PointSize"}, {3, "ClipDistance"}, {4, "CullDistance"}, {5, "VertexId"},
    {6, "InstanceId"}, {7, "PrimitiveId"}, {8, "InvocationId"}, {9, "Layer"}, {10, "ViewportIndex"},
    {11, "TessLevelOuter"}, {12, "TessLevelInner"}, {13, "TessCoord"}, {14, "PatchVertices"},
    {15, "FragCoord"}, {16, "PointCoord"}, {17, "FrontFacing"}, {18, "SampleId"}, {19, "SamplePosition"},
    {20, "SampleMask"}, {22, "FragDepth"}, {23, "HelperInvocation"}, {24, "NumWorkgroups"},
    {25, "WorkgroupSize"}, {26, "WorkgroupId"}, {27, "LocalInvocationId"}, {28, "GlobalInvocationId"},
    {29, "LocalInvocationIndex"}, {42, "VertexIndex"}, {43, "InstanceIndex"}};
const Name kSourceLang[] = {{0, "Unknown"}, {1, "ESSL"}, {2, "GLSL"}, {3, "OpenCL_C"}, {4, "OpenCL_CPP"},
                            {5, "HLSL"}};
const Name kFunctionControl[] = {{1, "Inline"}, {2, "DontInline"}, {4, "Pure"}, {8, "Const"}};
const Name kSelectionControl[] = {{1, "Flatten"}, {2, "DontFlatten"}};
const Name kLoopControl[] = {{1, "Unroll"}, {2, "DontUnroll"}};
const Name kMemoryAccess[] = {{1, "Volatile"}, {2, "Aligned"}, {4, "Nontemporal"}};
const Name kImageOperands[] = {{0x1, "Bias"},        {0x2, "Lod"},    {0x4, "Grad"},  {0x8, "ConstOffset"},
                               {0x10, "Offset"},     {0x20, "ConstOffsets"}, {0x40, "Sample"},
                               {0x80, "MinLod"}};
const Name kGlsl[] = {
    {1, "Round"}, {2, "RoundEven"}, {3, "Trunc"}, {4, "FAbs"}, {5, "SAbs"}, {6, "FSign"}, {7, "SSign"},
    {8, "Floor"}, {9, "Ceil"}, {10, "Fract"}, {11, "Radians"}, {12, "Degrees"}, {13, "Sin"}, {14, "Cos"},
    {15, "Tan"}, {16, "Asin"}, {17, "Acos"}, {18, "Atan"}, {19, "Sinh"}, {20, "Cosh"}, {21, "Tanh"},
    {22, "Asinh"}, {23, "Acosh"}, {24, "Atanh"}, {25, "Atan2"}, {26, "Pow"}, {27, "Exp"}, {28, "Log"},
    {29, "Exp2"}, {30, "Log2"}, {31, "Sqrt"}, {32, "InverseSqrt"}, {33, "Determinant"}, {34, "MatrixInverse"},
    {35, "Modf"}, {36, "ModfStruct"}, {37, "FMin"}, {38, "UMin"}, {39, "SMin"}, {40, "FMax"}, {41, "UMax"},
    {42, "SMax"}, {43, "FClamp"}, {44, "UClamp"}, {45, "SClamp"}, {46, "FMix"}, {47, "IMix"}, {48, "Step"},
    {49, "SmoothStep"}, {50, "Fma"}, {66, "Length"}, {67, "Distance"}, {68, "Cross"}, {69, "Normalize"},
    {70, "FaceForward"}, {71, "Reflect"}, {72, "Refract"}};

template <size_t N>
std::string enum_name(const Name (&t)[N], uint32_t v) {
  for (const Name& n : t)
    if (n.v == v) return n.n;
  return std::to_string(v);
}

template <size_t N>
std::string mask_name(const Name (&t)[N], uint32_t v) {
  if (v == 0) return "None";
  std::string s;
  for (const Name& n : t)
    if (v & n.v) {
      if (!s.empty()) s += "|";
      s += n.n;
      v &= ~n.v;
    }
  if (v) {
    if (!s.empty()) s += "|";
    char buf[16];
    std::snprintf(buf, sizeof buf, "0x%x", v);
    s += buf;
  }
  return s;
}

std::string id(uint32_t v) { return "%" + std::to_string(v); }

std::string hex8(uint32_t v) {
  char buf[16];
  std::snprintf(buf, sizeof buf, "0x%08X", v);
  return buf;
}

std::string quote(const std::string& s) {
  std::string r = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') r += '\\';
    r += c;
  }
  return r + "\"";
}

/* operands of a decoration after the decoration enumerant */
void decoration_operands(uint32_t dec, const std::vector<uint32_t>& ops, size_t i, std::string& s) {
  s += " " + enum_name(kDecoration, dec);
  if (dec == DecBuiltIn && i < ops.size()) {
    s += " " + enum_name(kBuiltIn, ops[i]);
    return;
  }
  for (; i < ops.size(); i++) s += " " + std::to_string(ops[i]);
}

struct DumpState {
  std::unordered_map<uint32_t, std::string> ext_sets;  /* result id -> extended instruction set name */
  std::unordered_map<uint32_t, uint32_t> int_width;    /* OpTypeInt result id -> width */
  std::unordered_map<uint32_t, uint32_t> type_of;      /* result id -> result type id */
};

std::string format_insn(const Insn& in, const DumpState& ds) {
  const auto& ext_sets = ds.ext_sets;
  const OpInfo* info = find_op(in.opcode);
  std::string name = info ? info->name : ("Op" + std::to_string(in.opcode));
  const auto& ops = in.ops;
  std::string lhs, rhs = name;
  size_t i = 0;
  auto take = [&](void) -> uint32_t { return i < ops.size() ? ops[i++] : 0u; };
  if (!info) {
    for (; i < ops.size(); i++) rhs += " " + std::to_string(ops[i]);
  } else if (std::strcmp(info->grammar, "*") == 0) {
    switch (in.opcode) {
      case OpExtInst: {
        uint32_t ty = take(), res = take(), set = take(), num = take();
        lhs = id(res);
        rhs += " " + id(ty) + " " + id(set);
        auto it = ext_sets.find(set);
        if (it != ext_sets.end() && it->second == "GLSL.std.450") rhs += " " + enum_name(kGlsl, num);
        else rhs += " " + std::to_string(num);
        for (; i < ops.size(); i++) rhs += " " + id(ops[i]);
        break;
      }
      case OpSpecConstantOp: {
        uint32_t ty = take(), res = take(), opc = take();
        lhs = id(res);
        const OpInfo* inner = find_op((uint16_t)opc);
        std::string iname = inner ? std::string(inner->name + 2) : std::to_string(opc);
        rhs += " " + id(ty) + " " + iname;
        for (; i < ops.size(); i++) rhs += " " + id(ops[i]);
        break;
      }
      case OpDecorate: {
        uint32_t target = take(), dec = take();
        rhs += " " + id(target);
        decoration_operands(dec, ops, i, rhs);
        break;
      }
      case OpMemberDecorate: {
        uint32_t target = take(), member = take(), dec = take();
        rhs += " " + id(target) + " " + std::to_string(member);
        decoration_operands(dec, ops, i, rhs);
        break;
      }
      case OpSwitch: {
        uint32_t sel = take(), def = take();
        rhs += " " + id(sel) + " " + id(def);
        uint32_t width = 32;
        auto ty = ds.type_of.find(sel);
        if (ty != ds.type_of.end()) {
          auto w = ds.int_width.find(ty->second);
          if (w != ds.int_width.end()) width = w->second;
        }
        while (i < ops.size()) {
          uint64_t lit = take();
          if (width > 32) lit |= (uint64_t)take() << 32;
          uint32_t target = take();
          rhs += " " + std::to_string(lit) + " " + id(target);
        }
        break;
      }
      default: break;
    }
  } else {
    const char* g = info->grammar;
    bool optional = false;
    while (*g) {
      char c = *g++;
      if (c == '?') {
        optional = true;
        continue;
      }
      if (i >= ops.size()) {
        if (optional || c == 'I' || c == 'L') break;
        break;
      }
      switch (c) {
        case 't': rhs += " " + id(take()); break;
        case 'r': lhs = id(take()); break;
        case 'i': rhs += " " + id(take()); break;
        case 'I':
          for (; i < ops.size(); i++) rhs += " " + id(ops[i]);
          break;
        case 'l': rhs += " " + std::to_string(take()); break;
        case 'L':
          for (; i < ops.size(); i++) rhs += " " + std::to_string(ops[i]);
          break;
        case 's': rhs += " " + quote(read_string(ops, i)); break;
        case 'c':
          for (; i < ops.size(); i++) rhs += " " + hex8(ops[i]);
          break;
        case 'e': {
          char k = *g++;
          uint32_t v = take();
          switch (k) {
            case 'C': rhs += " " + enum_name(kCapability, v); break;
            case 'A': rhs += " " + enum_name(kAddressing, v); break;
            case 'M': rhs += " " + enum_name(kMemoryModel, v); break;
            case 'X': rhs += " " + enum_name(kExecModel, v); break;
            case 'O': rhs += " " + enum_name(kExecMode, v); break;
            case 'S': rhs += " " + enum_name(kStorage, v); break;
            case 'F': rhs += " " + mask_name(kFunctionControl, v); break;
            case 'Q': rhs += " " + mask_name(kSelectionControl, v); break;
            case 'P': rhs += " " + mask_name(kLoopControl, v); break;
            case 'G': rhs += " " + enum_name(kSourceLang, v); break;
            case 'N': rhs += " " + mask_name(kMemoryAccess, v); break;
            case 'Y': rhs += " " + mask_name(kImageOperands, v); break;
            default: rhs += " " + std::to_string(v); break;
          }
          break;
        }
        default: break;
      }
    }
  }
  std::string out;
  if (!lhs.empty()) {
    if (lhs.size() < 12) out.append(12 - lhs.size(), ' ');
    out += lhs + " = " + rhs;
  } else {
    out.append(15, ' ');
    out += rhs;
  }
  return out;
}

}  // namespace

const char* opcode_name(uint16_t op) {
  const OpInfo* info = find_op(op);
  return info ? info->name : "OpUnknown";
}

std::string disassemble(const Module& m) {
  char buf[128];
  std::string out = "; SPIR-V\n";
  std::snprintf(buf, sizeof buf, "; Version: %u.%u\n", (m.version >> 16) & 0xFFu, (m.version >> 8) & 0xFFu);
  out += buf;
  std::snprintf(buf, sizeof buf, "; Generator: 0x%X\n; Bound: %u\n; Schema: %u\n", m.generator, m.bound, m.schema);
  out += buf;
  DumpState ds;
  for (const Insn& in : m.insns) {
    if (in.opcode == OpExtInstImport && !in.ops.empty()) {
      size_t i = 1;
      ds.ext_sets[in.ops[0]] = read_string(in.ops, i);
    }
    if (in.opcode == OpTypeInt && in.ops.size() >= 2) ds.int_width[in.ops[0]] = in.ops[1];
    const OpInfo* info = find_op(in.opcode);
    if (info && info->grammar[0] == 't' && info->grammar[1] == 'r' && in.ops.size() >= 2)
      ds.type_of[in.ops[1]] = in.ops[0];
    if ((in.opcode == OpExtInst || in.opcode == OpSpecConstantOp) && in.ops.size() >= 2)
      ds.type_of[in.ops[1]] = in.ops[0];
    out += format_insn(in, ds);
    std::snprintf(buf, sizeof buf, " ; 0x%08x\n", in.offset);
    out += buf;
  }
  return out;
}

}  // namespace spv
}  // namespace kz
