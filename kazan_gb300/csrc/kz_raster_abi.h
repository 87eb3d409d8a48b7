/*
 * kz_raster_abi.h - data shared by the host driver (C++) and the sm_103a pipeline kernels (CUDA).
 *
 * One command buffer is lowered into a table of draws (KzDraw), a table of pipelines (KzPipe) and a
 * list of raster segments (KzSegment).  A segment is a run of draws that render into one framebuffer
 * with a single raster mode; the kernels process one segment at a time:
 *
 * Opaque segments (visibility mode) resolve depth order-independently through a per-pixel 64-bit key
 * (depth, primitive sequence number) in HBM/L2:
 *   vis init  : per pixel     -> key of the loaded or cleared depth
 *   geometry  : per triangle  -> index fetch, position-only vertex shader (each vertex of a 256-triangle
 *                                chunk shaded once), clip, project, 16.8 snap, cull; small triangles are
 *                                rasterised on the spot into the keys (atomicMin), large ones become
 *                                records split into 8x8-pixel jobs
 *   large     : per job       -> warp-wide edge tests of one record over up to 16 blocks
 *   resolve   : per pixel     -> one fragment-shader call for the key's primitive, framebuffer store
 * Ordered segments (blending, discard, other compare ops) keep primitive order through screen tiles:
 *   geometry  : per triangle  -> KzTriRecord + screen-tile pair counts
 *   tile scan : per tile      -> exclusive prefix sum of the pair counts (bin offsets)
 *   bin       : per record    -> scatter the record index into every overlapped tile's bin
 *   raster    : per tile      -> bin sorted by primitive, per-pixel in-order depth test, blend, store
 *
 * The reference driver declares the entry points of this path but implements none of them
 * (vulkan-driver/src/api_impl.rs:4632-4653 vkCmdDraw/vkCmdDrawIndexed, :4780 vkCmdClearColorImage,
 * :3414 vkQueueSubmit); the layout below is this project's own.
 */
#ifndef KZ_RASTER_ABI_H
#define KZ_RASTER_ABI_H

#include <stdint.h>

#define KZ_MAX_VS_INPUTS 8         /* vertex attribute locations */
#define KZ_MAX_VARYINGS 16         /* scalar varyings (4 vec4 locations) */
#define KZ_MAX_BINDINGS 8
#define KZ_MAX_PIPES 8             /* distinct pipelines in one command buffer */
#define KZ_PUSH_BYTES 128          /* push constant block snapshot per draw */
#define KZ_GUARD_BAND 4.0f         /* clip-space guard band |x|,|y| <= 4 w */
#define KZ_SUBPIXEL_BITS 8         /* 16.8 fixed point */
#define KZ_MAX_CLIP_VERTS 9        /* 3 + one per clip plane */
#define KZ_DYN_SMEM (44 * 1024)    /* dynamic shared memory of the raster and persistent kernels */

/* vertex attribute formats the fetch understands */
enum KzAttrFormat {
  KZ_FMT_NONE = 0,
  KZ_FMT_F32x1 = 1,
  KZ_FMT_F32x2 = 2,
  KZ_FMT_F32x3 = 3,
  KZ_FMT_F32x4 = 4,
  KZ_FMT_U8x4_UNORM = 5,
  KZ_FMT_U32x1 = 6,
  KZ_FMT_U32x2 = 7,
  KZ_FMT_U32x3 = 8,
  KZ_FMT_U32x4 = 9
};

/* raster modes of a segment */
enum KzRasterMode {
  KZ_MODE_VISIBILITY = 0, /* order-independent depth resolve (opaque, no blend, no discard) */
  KZ_MODE_ORDERED = 1     /* per-pixel in-order processing (blending, discard, any compare op) */
};

/* what the key of the visibility resolve encodes */
enum KzVisKey {
  KZ_VIS_LESS = 0,     /* min (z, g+1): earliest wins ties */
  KZ_VIS_LEQUAL = 1,   /* min (z, ~g): latest wins ties */
  KZ_VIS_GREATER = 2,  /* min (~z, g+1) */
  KZ_VIS_GEQUAL = 3,   /* min (~z, ~g) */
  KZ_VIS_LAST = 4      /* depth test off: latest fragment wins */
};

/* attachment load ops as the tiles see them */
enum KzLoad { KZ_LOAD_LOAD = 0, KZ_LOAD_CLEAR = 1, KZ_LOAD_DONT_CARE = 2 };

/* colour formats the raster stores.  The sRGB formats hold the 8-bit sRGB codes of the red, green and
 * blue channels (encoded at store, decoded before blending, kz_srgb_table.h) and a linear alpha. */
enum KzColorFormat {
  KZ_CF_NONE = 0,
  KZ_CF_RGBA8 = 1,
  KZ_CF_BGRA8 = 2,
  KZ_CF_RGBA8_SRGB = 3,
  KZ_CF_BGRA8_SRGB = 4
};

/* depth attachment formats.  D16 and D24 depths are compared and stored as rint(z * (2^bits - 1)), an
 * integer the kernels hold in a float (exact below 2^24); D24S8 texels keep the depth in bits 0..23 and
 * the stencil in bits 24..31.  Only ordered segments render into D16 / D24S8. */
enum KzDepthFormat { KZ_DF_D32 = 0, KZ_DF_D16 = 1, KZ_DF_D24S8 = 2 };

typedef struct KzAttr {
  uint32_t location;
  uint32_t binding;
  uint32_t format; /* KzAttrFormat */
  uint32_t offset;
} KzAttr;

/* fixed-function + shader selection of one pipeline (device copy) */
typedef struct KzPipe {
  uint32_t num_attrs;
  uint32_t pos_input_mask;    /* locations the position-only vertex shader reads */
  uint32_t full_input_mask;   /* locations the full vertex shader reads */
  uint32_t num_varyings;      /* scalars written by the vertex shader and read by the fragment shader */
  KzAttr attrs[KZ_MAX_VS_INPUTS];
  uint32_t binding_stride[KZ_MAX_BINDINGS];
  uint32_t binding_instanced; /* bit b: binding b advances per instance */
  uint32_t flat_mask;         /* bit k: varying k is flat */
  uint32_t noperspective_mask;/* bit k: varying k is linear in screen space */
  uint32_t cull_mode;         /* VkCullModeFlags */
  uint32_t front_ccw;         /* 1 if VK_FRONT_FACE_COUNTER_CLOCKWISE */
  uint32_t depth_test, depth_write, depth_compare; /* VkCompareOp */
  uint32_t blend_enable;
  uint32_t src_color, dst_color, color_op, src_alpha, dst_alpha, alpha_op; /* VkBlendFactor / VkBlendOp */
  uint32_t write_mask;        /* VkColorComponentFlags */
  uint32_t fs_discards;
  uint32_t has_fs;
  float blend_const[4];       /* VkPipelineColorBlendStateCreateInfo::blendConstants (draws carry their own copy) */
  uint32_t fs_passthrough;    /* the fragment shader only copies varyings 0..3 to colour components 0..3 */
  uint32_t stencil_test;      /* VkPipelineDepthStencilStateCreateInfo::stencilTestEnable */
  /* front and back VkStencilOpState, two words each: failOp | passOp << 3 | depthFailOp << 6 | compareOp << 9,
   * then compareMask | writeMask << 8 | reference << 16 */
  uint32_t stencil[4];
  uint32_t pad;
} KzPipe;

/* one recorded draw (instances expanded by the kernels) */
typedef struct KzDraw {
  uint64_t vb[KZ_MAX_BINDINGS]; /* device address of each bound vertex buffer (buffer + offset) */
  uint64_t ib;                  /* device address of index 0 of this draw (buffer + offset + firstIndex*size) */
  uint32_t indexed;             /* 0: vkCmdDraw, 1: u32 indices, 2: u16 indices */
  int32_t vertex_offset;        /* vkCmdDrawIndexed vertexOffset, or vkCmdDraw firstVertex */
  uint32_t first_instance;
  uint32_t instance_count;
  uint32_t tri_count;           /* triangles per instance */
  uint32_t pipe;                /* index into the pipeline table */
  uint32_t prim_base;           /* primitive sequence number of its first triangle within the segment */
  uint32_t push_index;          /* index of its push-constant snapshot */
  /* viewport transform constants: xf = fma(xd, hx, ox), yf = fma(yd, hy, oy), zf = fma(zd, pz, oz) */
  float hx, ox, hy, oy, pz, oz, zmin, zmax;
  int32_t rect[4];              /* pixel rectangle x0,y0,x1,y1 (exclusive): fb & render area & scissor & viewport */
  /* indirect draws (vkCmdDrawIndirect / vkCmdDrawIndexedIndirect): kz_k_indirect reads the command at
   * `indirect` and writes ib, vertex_offset, first_instance, instance_count, tri_count, prim_base and
   * chunk_base before the segment runs */
  uint64_t indirect;            /* device address of a VkDrawIndirectCommand / VkDrawIndexedIndirectCommand; 0: direct */
  uint64_t ib_base;             /* indexed: device address of index 0 of the bound index buffer (buffer + offset) */
  uint32_t elem_limit;          /* indices the bound index buffer holds past ib_base (indexed), or vertices every
                                   per-vertex binding holds (non-indexed); a command beyond it is skipped */
  uint32_t instance_limit;      /* instances every per-instance binding holds */
  uint32_t chunk_base;          /* first chunk of the draw within its segment */
  uint32_t call_index;          /* position of the command within its vkCmdDraw*Indirect*Count call */
  uint64_t count_addr;          /* vkCmdDraw*IndirectCount: device address of the u32 draw count (the draw is
                                   skipped when call_index >= count); 0: every recorded command draws */
  uint32_t samples;             /* rasterizationSamples of its pass: 1, or 4 (KZ_MS_* positions) */
  uint32_t pad;
  uint32_t stencil[4];          /* the draw's stencil state in KzPipe::stencil's encoding: the pipeline's, with
                                   vkCmdSetStencilCompareMask / WriteMask / Reference applied where dynamic */
  float blend_const[4];         /* the blend constants in effect at the draw (the pipeline's, or
                                   vkCmdSetBlendConstants where dynamic), clamped to [0, 1] */
} KzDraw;

/* the four sample positions of a 4x multisampled pixel (the Vulkan standard positions), in 1/256 pixel
 * from the pixel's corner: (96, 32), (224, 96), (32, 160), (160, 224) */
#define KZ_MS_SAMPLES 4
#define KZ_MS_LO 32   /* smallest sample offset in either axis */
#define KZ_MS_HI 224  /* largest */

/* geometry work unit: a contiguous run of at most KZ_CHUNK triangles of one draw */
#define KZ_CHUNK 256
typedef struct KzChunk {
  uint32_t draw;   /* index into the draw table */
  uint32_t first;  /* first triangle (instance-major index within the draw) */
  uint32_t count;
  uint32_t pad;
} KzChunk;

/* one oriented, snapped, visible (sub-)triangle */
typedef struct KzTriRecord {
  int32_t x[3], y[3];   /* 16.8 framebuffer coordinates, oriented so that the signed area S > 0 */
  float z0, dz1, dz2;   /* depth: z0, z1 - z0, z2 - z0 */
  float inv_s;          /* 1 / (float)S */
  uint32_t g;           /* primitive sequence number within the segment (API order) */
  uint32_t info;        /* bit 0..2 top-left flags of edges 0,1,2; bit 3 swapped; bits 4..7 clip sub-triangle
                           index + 1 (0 = not clipped); bit 8 front facing */
  uint32_t bb0;         /* bounding box (inclusive pixels): x0 | y0 << 16 */
  uint32_t bb1;         /* x1 | y1 << 16 */
  uint32_t draw;        /* draw index (absolute) */
  uint32_t pad;
} KzTriRecord;          /* 64 bytes */

/* per-segment scratch counters (zeroed before the segment runs) */
typedef struct KzSegCounters {
  uint32_t rec_count;   /* records written (visibility mode: large triangles only) */
  uint32_t pair_count;  /* (tile, record) pairs (visibility mode: large-triangle jobs) */
  uint32_t geom_next;   /* work-stealing cursor over chunks */
  uint32_t bin_next;    /* work-stealing cursor over records */
  uint32_t tile_next;   /* work-stealing cursor over tiles */
  uint32_t fragments;   /* statistics: covered fragments (visibility mode counts depth-pass candidates) */
  uint32_t max_bin;     /* largest bin */
  uint32_t large_done;  /* per-draw launches: large-triangle jobs the earlier kz_k_vis_large launches processed */
  uint32_t large_blocks;/* per-draw launches: blocks of the current kz_k_vis_large launch that have finished */
  uint32_t pad[2];
} KzSegCounters;

typedef struct KzSegment {
  uint32_t first_draw, num_draws;
  uint32_t first_chunk, num_chunks;
  uint32_t num_prims;        /* total triangles (all instances) */
  uint32_t mode;             /* KzRasterMode */
  uint32_t vis_key;          /* KzVisKey (visibility mode) */
  uint32_t tile;             /* tile side in pixels: 8, 16, 32 or 64 */
  uint32_t tiles_x, tiles_y;
  /* framebuffer */
  uint64_t color;            /* device address of the colour attachment (0 if none) */
  uint64_t depth;            /* device address of the D32 attachment (0 if none) */
  uint32_t width, height;
  uint32_t color_pitch;      /* bytes per row */
  uint32_t depth_pitch;
  uint32_t color_format;     /* KzColorFormat */
  uint32_t color_load, depth_load;  /* KzLoad */
  uint32_t color_store, depth_store;/* 1: store, 0: discard */
  uint32_t clear_color;      /* packed RGBA8 of the clear value in attachment byte order */
  float clear_depth;
  int32_t area[4];           /* render area x0,y0,x1,y1 (exclusive) */
  /* scratch */
  uint64_t records;          /* KzTriRecord[rec_cap] */
  uint64_t tile_count;       /* u32[tiles] */
  uint64_t tile_offset;      /* u32[tiles + 1] */
  uint64_t tile_cursor;      /* u32[tiles] */
  uint64_t tile_order;       /* u32[tiles]: the tiles by decreasing bin size (powers of two), for the raster */
  uint64_t bins;             /* u32[pair_cap] */
  uint64_t counters;         /* KzSegCounters* */
  uint64_t vis;              /* visibility mode: u64 (depth, primitive) key per pixel, width * height */
  uint32_t rec_cap, pair_cap;
  uint32_t segment_index;
  uint32_t shade_stride;     /* ordered mode: bytes per record in `shades` */
  uint64_t shades;           /* ordered mode: per record, the shading setup of an unclipped triangle:
                                float 1/w[3], pad, then varyings (divided by w unless flat/noperspective)
                                [3][num_varyings] */
  uint64_t draw_lut;         /* u32 per 256 primitives: the draw holding primitive 256 i (0: search) */
  uint32_t indirect;         /* 1: every draw is indirect; kz_k_indirect writes num_chunks and num_prims, and
                                chunk k belongs to the last draw whose chunk_base <= k (no KzChunk entries) */
  uint32_t chunk_cap;        /* indirect: entries of chunk_table */
  uint64_t chunk_table;      /* indirect: KzChunk per chunk (kz_k_indirect_tables); used when
                                num_chunks <= chunk_cap, else chunk_at searches the draws */
  uint64_t lut_table;        /* indirect: room for the draw lookup; kz_k_indirect points draw_lut at it when
                                the segment's primitives need at most lut_cap entries, else sets it to 0 */
  uint32_t lut_cap;
  uint32_t depth_format;     /* KzDepthFormat; clear_depth holds the converted value for D16 / D24S8 */
  uint32_t stencil_load;     /* KzLoad of the stencil aspect (D24S8) */
  uint32_t clear_stencil;
  uint32_t samples;          /* 1, or 4: colour and depth texels hold KZ_MS_SAMPLES samples each, sample s of
                                pixel x at byte 16 x + 4 s of its row (ordered segments, D32 depth, tiles <= 16) */
  uint32_t pad2;
  /* ordered segments raster by kz_k_raster_direct: device addresses of the TMA tensor maps (CUtensorMap, 128
   * bytes, 64-byte aligned) of the colour and depth attachments -- 32-bit texels, width x height, box of
   * tile x tile texels -- or 0 where the tile is read and written with plain loads and stores */
  uint64_t tmap_color, tmap_depth;
} KzSegment;

/* status words written by the kernels (one per submission) */
enum KzStatusBits {
  KZ_STATUS_OK = 0,
  KZ_STATUS_RECORD_OVERFLOW = 1,
  KZ_STATUS_PAIR_OVERFLOW = 2,
  KZ_STATUS_BARRIER_TIMEOUT = 4,
  KZ_STATUS_BIN_TOO_LARGE = 8,
  KZ_STATUS_INDIRECT_RANGE = 16,  /* an indirect command reads past its bound buffers: that draw was skipped */
  KZ_STATUS_INDIRECT_LIMIT = 32,  /* an indirect segment's triangles reach 2^32: the segment was skipped */
  KZ_STATUS_TMA_TIMEOUT = 64      /* a tile's tensor copy did not complete within its wait limit */
};

typedef struct KzStatus {
  uint32_t flags;            /* KzStatusBits */
  uint32_t failed_segment;   /* first segment whose raster was skipped */
  uint32_t need_records;     /* largest record count any segment asked for */
  uint32_t need_pairs;       /* largest pair count any segment asked for */
  uint32_t barrier_arrive;   /* grid barrier state (persistent kernel) */
  uint32_t barrier_gen;
  uint32_t fragments_lo;     /* statistics */
  uint32_t pad;
} KzStatus;

/* the whole lowered command buffer as the kernels see it */
typedef struct KzFrame {
  uint64_t draws;            /* KzDraw[] */
  uint64_t pipes;            /* KzPipe[] */
  uint64_t chunks;           /* KzChunk[] */
  uint64_t segments;         /* KzSegment[] */
  uint64_t push;             /* uint8_t[num_push][KZ_PUSH_BYTES] */
  uint64_t status;           /* KzStatus* */
  uint32_t num_segments;
  uint32_t first_segment;    /* segments before it are skipped (restart after an overflow) */
  /* one launch of the geometry kernels processes chunks [chunk_begin, min(chunk_end, num_chunks)) of its
   * segment: all of them (0, ~0u), or one draw's in the per-draw launch form */
  uint32_t chunk_begin, chunk_end;
  uint32_t jobs_incremental; /* kz_k_vis_large: process only the jobs added since the previous launch for
                                this segment (per-draw launch form), else all of the segment's jobs */
  uint32_t barrier_ns;       /* persistent kernels: a grid barrier gives up (KZ_STATUS_BARRIER_TIMEOUT) after
                                waiting this many nanoseconds */
  uint32_t warp_px;          /* visibility path: unclipped triangles whose boxes hold at most this many pixels
                                are rasterised by their geometry warp, larger ones become jobs */
  uint32_t job_blocks;       /* visibility path: 8x8 pixel blocks per large-triangle job, 1..32 */
} KzFrame;

#define KZ_WARP_PX_DEFAULT 192
#define KZ_JOB_BLOCKS_DEFAULT 16

/* --- shader call ABI (kernels <-> JIT-linked shader device functions) --- */

typedef struct KzVsIn {
  float attr[KZ_MAX_VS_INPUTS][4];
  uint32_t vertex_index;
  uint32_t instance_index;
  uint32_t pad[2];
} KzVsIn; /* 144 bytes */

typedef struct KzVsOut {
  float pos[4];
  float var[KZ_MAX_VARYINGS];
} KzVsOut; /* 80 bytes */

typedef struct KzFsIn {
  float var[KZ_MAX_VARYINGS];
  float frag_coord[4];
  uint32_t front_facing;
  uint32_t pad[3];
} KzFsIn; /* 96 bytes */

typedef struct KzFsOut {
  float color[4];
  uint32_t discard;
  uint32_t pad[3];
} KzFsOut; /* 32 bytes */

/* --- descriptors (vkUpdateDescriptorSets / vkCmdBindDescriptorSets) ---
 * A draw's snapshot in the push area is its KZ_PUSH_BYTES of push constants followed by one KzDescriptor
 * per descriptor slot of its pipeline layout (sets in order, bindings in increasing binding number, array
 * elements in order), so every shader function reaches them through its `push` argument. */
#define KZ_DESC_OFFSET KZ_PUSH_BYTES  /* byte offset of slot 0 within a draw's snapshot */
#define KZ_MAX_DESC_SETS 4
#define KZ_MAX_DESC_BINDINGS 16       /* binding numbers 0..15 in each set */
#define KZ_MAX_DESC_SLOTS 64          /* descriptor slots of one pipeline layout */

typedef struct KzDescriptor {
  uint64_t addr;     /* uniform buffer: device address of the bound range (offset and dynamic offset applied);
                        combined image sampler: device address of texel (0, 0) */
  uint32_t range;    /* uniform buffer: bytes of the bound range */
  uint32_t width, height;
  uint32_t pitch;    /* image: bytes per row */
  uint32_t format;   /* image: KzColorFormat of the texels (RGBA8 or BGRA8, UNORM) */
  uint32_t sampler;  /* KzSamplerBits */
} KzDescriptor;      /* 32 bytes */

/* sampler state packed into KzDescriptor::sampler */
enum KzSamplerBits {
  KZ_SAMP_LINEAR = 1u,         /* VK_FILTER_LINEAR (else NEAREST); the sampler's min and mag filters agree */
  KZ_SAMP_UNNORMALIZED = 2u,   /* unnormalizedCoordinates */
  KZ_SAMP_ADDR_U_SHIFT = 4,    /* bits 4..6: VkSamplerAddressMode for u */
  KZ_SAMP_ADDR_V_SHIFT = 8,    /* bits 8..10: for v */
  KZ_SAMP_BORDER_SHIFT = 12    /* bits 12..13: 0 transparent black, 1 opaque black, 2 opaque white */
};

#endif /* KZ_RASTER_ABI_H */
