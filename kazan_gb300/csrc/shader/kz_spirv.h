/*
 * kz_spirv.h - SPIR-V binary decoding for the shader path.
 *
 * Plays the role of the reference's generated decoder (spirv-parser/src/generated_parser.rs, entry
 * points `convert_bytes_to_words` and `Parser::start`) for the subset of the SPIR-V 1.x grammar that
 * graphics shaders use.  Opcode, enumerant and extended-instruction numbers are the ones the SPIR-V
 * and GLSL.std.450 specifications assign.  `disassemble` prints the same text form as the reference's
 * `Display` implementations (header block, right-aligned result ids, hex literals for constants,
 * " ; 0x<byte offset>" suffix) so the decoder can be checked against the reference's golden dumps
 * (spirv-parser/src/lib.rs:45-216).
 */
#ifndef KZ_SPIRV_H
#define KZ_SPIRV_H

#include <cstdint>
#include <string>
#include <vector>

namespace kz {
namespace spv {

constexpr uint32_t kMagic = 0x07230203u;

enum Op : uint16_t {
  OpNop = 0, OpUndef = 1, OpSourceContinued = 2, OpSource = 3, OpSourceExtension = 4, OpName = 5,
  OpMemberName = 6, OpString = 7, OpLine = 8, OpExtension = 10, OpExtInstImport = 11, OpExtInst = 12,
  OpMemoryModel = 14, OpEntryPoint = 15, OpExecutionMode = 16, OpCapability = 17, OpTypeVoid = 19,
  OpTypeBool = 20, OpTypeInt = 21, OpTypeFloat = 22, OpTypeVector = 23, OpTypeMatrix = 24, OpTypeImage = 25,
  OpTypeSampler = 26, OpTypeSampledImage = 27, OpTypeArray = 28, OpTypeRuntimeArray = 29, OpTypeStruct = 30,
  OpTypeOpaque = 31, OpTypePointer = 32, OpTypeFunction = 33, OpConstantTrue = 41, OpConstantFalse = 42,
  OpConstant = 43, OpConstantComposite = 44, OpConstantSampler = 45, OpConstantNull = 46,
  OpSpecConstantTrue = 48, OpSpecConstantFalse = 49, OpSpecConstant = 50, OpSpecConstantComposite = 51,
  OpSpecConstantOp = 52, OpFunction = 54, OpFunctionParameter = 55, OpFunctionEnd = 56, OpFunctionCall = 57,
  OpVariable = 59, OpImageTexelPointer = 60, OpLoad = 61, OpStore = 62, OpCopyMemory = 63,
  OpAccessChain = 65, OpInBoundsAccessChain = 66, OpPtrAccessChain = 67, OpDecorate = 71,
  OpMemberDecorate = 72, OpVectorExtractDynamic = 77, OpVectorInsertDynamic = 78, OpVectorShuffle = 79,
  OpCompositeConstruct = 80, OpCompositeExtract = 81, OpCompositeInsert = 82, OpCopyObject = 83,
  OpTranspose = 84, OpSampledImage = 86, OpImageSampleImplicitLod = 87, OpImageSampleExplicitLod = 88,
  OpImageSampleProjImplicitLod = 91, OpImageSampleProjExplicitLod = 92, OpImageFetch = 95, OpImage = 100,
  OpImageQuerySizeLod = 103, OpImageQuerySize = 104,
  OpConvertFToU = 109, OpConvertFToS = 110, OpConvertSToF = 111, OpConvertUToF = 112, OpUConvert = 113,
  OpSConvert = 114, OpFConvert = 115, OpBitcast = 124, OpSNegate = 126, OpFNegate = 127, OpIAdd = 128,
  OpFAdd = 129, OpISub = 130, OpFSub = 131, OpIMul = 132, OpFMul = 133, OpUDiv = 134, OpSDiv = 135,
  OpFDiv = 136, OpUMod = 137, OpSRem = 138, OpSMod = 139, OpFRem = 140, OpFMod = 141,
  OpVectorTimesScalar = 142, OpMatrixTimesScalar = 143, OpVectorTimesMatrix = 144, OpMatrixTimesVector = 145,
  OpMatrixTimesMatrix = 146, OpOuterProduct = 147, OpDot = 148, OpAny = 154, OpAll = 155, OpIsNan = 156,
  OpIsInf = 157, OpLogicalEqual = 164, OpLogicalNotEqual = 165, OpLogicalOr = 166, OpLogicalAnd = 167,
  OpLogicalNot = 168, OpSelect = 169, OpIEqual = 170, OpINotEqual = 171, OpUGreaterThan = 172,
  OpSGreaterThan = 173, OpUGreaterThanEqual = 174, OpSGreaterThanEqual = 175, OpULessThan = 176,
  OpSLessThan = 177, OpULessThanEqual = 178, OpSLessThanEqual = 179, OpFOrdEqual = 180, OpFUnordEqual = 181,
  OpFOrdNotEqual = 182, OpFUnordNotEqual = 183, OpFOrdLessThan = 184, OpFUnordLessThan = 185,
  OpFOrdGreaterThan = 186, OpFUnordGreaterThan = 187, OpFOrdLessThanEqual = 188, OpFUnordLessThanEqual = 189,
  OpFOrdGreaterThanEqual = 190, OpFUnordGreaterThanEqual = 191, OpShiftRightLogical = 194,
  OpShiftRightArithmetic = 195, OpShiftLeftLogical = 196, OpBitwiseOr = 197, OpBitwiseXor = 198,
  OpBitwiseAnd = 199, OpNot = 200, OpBitFieldInsert = 201, OpBitFieldSExtract = 202, OpBitFieldUExtract = 203,
  OpBitReverse = 204, OpBitCount = 205, OpDPdx = 207, OpDPdy = 208, OpFwidth = 209, OpPhi = 245,
  OpLoopMerge = 246, OpSelectionMerge = 247, OpLabel = 248, OpBranch = 249, OpBranchConditional = 250,
  OpSwitch = 251, OpKill = 252, OpReturn = 253, OpReturnValue = 254, OpUnreachable = 255,
  OpModuleProcessed = 330
};

enum Decoration : uint32_t {
  DecRelaxedPrecision = 0, DecSpecId = 1, DecBlock = 2, DecBufferBlock = 3, DecRowMajor = 4, DecColMajor = 5,
  DecArrayStride = 6, DecMatrixStride = 7, DecBuiltIn = 11, DecNoPerspective = 13, DecFlat = 14,
  DecCentroid = 16, DecSample = 17, DecInvariant = 18, DecLocation = 30, DecComponent = 31, DecIndex = 32,
  DecBinding = 33, DecDescriptorSet = 34, DecOffset = 35, DecNoContraction = 42
};

enum BuiltIn : uint32_t {
  BuiltInPosition = 0, BuiltInPointSize = 1, BuiltInClipDistance = 3, BuiltInCullDistance = 4,
  BuiltInVertexId = 5, BuiltInInstanceId = 6, BuiltInFragCoord = 15, BuiltInFrontFacing = 17,
  BuiltInFragDepth = 22, BuiltInVertexIndex = 42, BuiltInInstanceIndex = 43
};

enum StorageClass : uint32_t {
  SCUniformConstant = 0, SCInput = 1, SCUniform = 2, SCOutput = 3, SCWorkgroup = 4, SCCrossWorkgroup = 5,
  SCPrivate = 6, SCFunction = 7, SCGeneric = 8, SCPushConstant = 9, SCAtomicCounter = 10, SCImage = 11,
  SCStorageBuffer = 12
};

enum ExecutionModel : uint32_t {
  EMVertex = 0, EMTessellationControl = 1, EMTessellationEvaluation = 2, EMGeometry = 3, EMFragment = 4,
  EMGLCompute = 5, EMKernel = 6
};

enum ExecutionMode : uint32_t { ModeOriginUpperLeft = 7, ModeOriginLowerLeft = 8, ModeEarlyFragmentTests = 9,
  ModeDepthReplacing = 12, ModeLocalSize = 17 };

/* GLSL.std.450 extended instructions */
enum GLSLstd450 : uint32_t {
  GRound = 1, GRoundEven = 2, GTrunc = 3, GFAbs = 4, GSAbs = 5, GFSign = 6, GSSign = 7, GFloor = 8, GCeil = 9,
  GFract = 10, GRadians = 11, GDegrees = 12, GSin = 13, GCos = 14, GTan = 15, GAsin = 16, GAcos = 17,
  GAtan = 18, GSinh = 19, GCosh = 20, GTanh = 21, GAsinh = 22, GAcosh = 23, GAtanh = 24, GAtan2 = 25,
  GPow = 26, GExp = 27, GLog = 28, GExp2 = 29, GLog2 = 30, GSqrt = 31, GInverseSqrt = 32, GDeterminant = 33,
  GMatrixInverse = 34, GModf = 35, GModfStruct = 36, GFMin = 37, GUMin = 38, GSMin = 39, GFMax = 40,
  GUMax = 41, GSMax = 42, GFClamp = 43, GUClamp = 44, GSClamp = 45, GFMix = 46, GIMix = 47, GStep = 48,
  GSmoothStep = 49, GFma = 50, GFrexp = 51, GFrexpStruct = 52, GLdexp = 53, GPackSnorm4x8 = 54,
  GPackUnorm4x8 = 55, GPackSnorm2x16 = 56, GPackUnorm2x16 = 57, GPackHalf2x16 = 58, GUnpackSnorm2x16 = 60,
  GUnpackUnorm2x16 = 61, GUnpackHalf2x16 = 62, GUnpackSnorm4x8 = 63, GUnpackUnorm4x8 = 64, GLength = 66,
  GDistance = 67, GCross = 68, GNormalize = 69, GFaceForward = 70, GReflect = 71, GRefract = 72, GFindILsb = 73,
  GFindSMsb = 74, GFindUMsb = 75, GNMin = 79, GNMax = 80, GNClamp = 81
};

struct Insn {
  uint16_t opcode = 0;
  uint32_t offset = 0;             /* byte offset of the instruction in the module */
  std::vector<uint32_t> ops;       /* operand words (everything after the first word) */
};

struct Module {
  uint32_t version = 0, generator = 0, bound = 0, schema = 0;
  std::vector<Insn> insns;
};

/* decode a module; returns an empty string on success, else a message */
std::string decode(const uint32_t* words, size_t count, Module& out);
/* bytes -> words (little endian, length must be a multiple of 4) */
bool bytes_to_words(const uint8_t* bytes, size_t n, std::vector<uint32_t>& words);
/* text dump (see the header comment) */
std::string disassemble(const Module& m);
/* a literal string operand starting at ops[i]; advances i past it */
std::string read_string(const std::vector<uint32_t>& ops, size_t& i);
const char* opcode_name(uint16_t op);

}  // namespace spv
}  // namespace kz

#endif
