/* phe_gb300.h - C ABI of the GB300 ray-cast and wavefront-shading core.
 *
 * A drop-in for the ray-cast path of PetorSFZ/PhantasyEngineTestbed. All structs are
 * byte-identical to the reference's (static_asserts in the implementation); all entry points
 * return a phe_status and never abort; phe_last_error() describes the last failure on the
 * calling thread. Device pointers are plain CUDA device addresses; `stream` is a cudaStream_t
 * (NULL = legacy default stream). Launch functions are asynchronous on `stream` unless stated.
 *
 * Reference paths below are relative to the reference project root.
 */
#ifndef PHE_GB300_H
#define PHE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------------
 * Status codes. The reference has none (CHECK_CUDA_ERROR logs and continues,
 * source/cuda_ray_tracer/CudaHelpers.hpp:13-25); every function here returns one of these.
 * ------------------------------------------------------------------------------------------- */
typedef int phe_status;
#define PHE_OK 0
#define PHE_ERR_INVALID_ARGUMENT 1   /* null pointer, zero size where not allowed, bad enum */
#define PHE_ERR_INVALID_SCENE 2      /* BVH fails validation (index out of range, cycle, too deep) */
#define PHE_ERR_CUDA 3               /* a CUDA runtime call failed; text in phe_last_error() */
#define PHE_ERR_OUT_OF_MEMORY 4      /* device or host allocation failed */
#define PHE_ERR_BUDGET 5             /* admission refused: device-memory budget exhausted */
#define PHE_ERR_TIMEOUT 6            /* a bounded device-side wait ran out */
#define PHE_ERR_NOT_FOUND 7          /* unknown scene / request id */
#define PHE_ERR_TOO_LARGE 8          /* size beyond a documented maximum */
#define PHE_ERR_NOT_READY 9          /* result not available yet (poll again) */
#define PHE_ERR_NO_DEVICE 10         /* no CUDA device is visible */
#define PHE_ERR_CANCELLED 11         /* the request was cancelled before it was admitted */

/* ---------------------------------------------------------------------------------------------
 * Layouts (byte-identical to the reference)
 * ------------------------------------------------------------------------------------------- */

/* phe::BVHNode, source/phantasy_engine/ray_tracer_common/BVHNode.hpp:23-149 (64 bytes).
 * fData = [lc.min.xyz, lc.max.x] [lc.max.yz, rc.min.xy] [rc.min.z, rc.max.xyz];
 * iData = [lcIndex, rcIndex, lcNumTriangles, rcNumTriangles]; a leaf child has a non-zero
 * triangle count and a bitwise-negated (~) first-slot index; node 0 is the root. */
typedef struct phe_bvh_node { float fData[12]; int32_t iData[4]; } phe_bvh_node;

/* phe::TriangleVertices, ray_tracer_common/Triangle.hpp:17-23 (48 bytes). The .w lanes are
 * 0, or -1 on the last triangle of each leaf (StaticBVHBuilder.cpp:33-45). */
typedef struct phe_triangle_vertices { float v0[4]; float v1[4]; float v2[4]; } phe_triangle_vertices;

/* phe::TriangleData, ray_tracer_common/Triangle.hpp:25-37 (64 bytes), same slot order. */
typedef struct phe_triangle_data {
	float n0[3], n1[3], n2[3];
	float uv0[2], uv1[2], uv2[2];
	uint32_t materialIndex;
} phe_triangle_data;

/* phe::RayIn, cuda_ray_tracer/kernels/RayCastKernel.hpp:22-37 (32 bytes):
 * data1 = (origin.xyz, tMin), data2 = (dir.xyz, tMax). */
typedef struct phe_ray_in { float data1[4]; float data2[4]; } phe_ray_in;

/* phe::RayHit, cuda_ray_tracer/kernels/RayCastKernel.hpp:39-45 (16 bytes).
 * Hit: triangleIndex = slot index, t, barycentric u, v. Miss: triangleIndex = ~0u, t = the ray's
 * tMax (as rayCastKernel, RayCastKernel.cu:396-409), u = v = 0 (the reference leaves them unset).
 * A hit is accepted when tMin <= t < tMax (exclusive tMax, RayCastKernel.cu:361). */
typedef struct phe_ray_hit { uint32_t triangleIndex; float t; float u; float v; } phe_ray_hit;

/* phe::CameraDef, ray_tracer_common/GenerateRays.hpp:14-24. */
typedef struct phe_camera_def { float origin[3]; float dir[3]; float dX[3]; float dY[3]; } phe_camera_def;

/* The shading inputs of phe::SphereLight (level/SphereLight.hpp:13-26). */
typedef struct phe_sphere_light {
	float pos[3]; float radius; float range; float strength[3]; int32_t staticShadows;
} phe_sphere_light;

/* Material (rendering/Material.hpp:17-55, byte-identical to the reference's Material: iData, fData1,
 * fData2): texture indices of albedo, roughness and metallic (-1 = none; the fourth is unused),
 * albedo rgba, roughness, metallic, two unused floats. A texture replaces its constant. */
typedef struct phe_material {
	int32_t texIndex[4];
	float albedo[4];
	float roughness;
	float metallic;
	float pad[2];
} phe_material;

/* A texture in the reference's RawImage form (rendering/RawImage.hpp:21-28): 8-bit channels, 1, 2 or
 * 4 bytes per pixel, rows `pitch` bytes apart starting with row 0 (texel y = 0). Host memory. */
typedef struct phe_texture {
	const uint8_t* data;
	int32_t width, height;   /* 1 .. 65536 */
	uint32_t bytesPerPixel;  /* 1, 2 or 4 */
	uint32_t pitch;          /* >= width * bytesPerPixel */
} phe_texture;

/* ---------------------------------------------------------------------------------------------
 * Library
 * ------------------------------------------------------------------------------------------- */

/* Version as 10000*major + 100*minor + patch. */
int phe_version(void);
/* Text of the last error on this thread ("" if none). The pointer stays valid until the next
 * call on this thread. */
const char* phe_last_error(void);

/* ---------------------------------------------------------------------------------------------
 * Host-side scene tools (no GPU needed)
 * ------------------------------------------------------------------------------------------- */

/* Synthetic scene recipe: an N x N-cell heightfield (2 triangles per cell, height = sum of 4
 * seeded sine octaves) plus `numCubes` cubes resting on it; the world is scaled by N/64 so the
 * cell size stays 1/64 (keeps the reference's absolute 1e-5 determinant epsilon,
 * Intersection.hpp:28, far from the triangle scale). Materials: one per triangle, albedo
 * U[0.2, 0.8] per channel, roughness 1, metallic 0. */
typedef struct phe_scene_recipe {
	uint32_t gridCells;      /* N */
	uint32_t numCubes;
	int32_t rotatedCubes;    /* 0 = axis-aligned, 1 = uniformly random rotation */
	uint32_t pad;
	uint64_t seed;
} phe_scene_recipe;
/* Triangle count of a recipe (2*N*N + 12*numCubes). */
uint64_t phe_scene_recipe_triangles(const phe_scene_recipe* recipe);
/* Writes `triVerts` (9 floats per triangle: v0 v1 v2), `datas` (flat normals, zero uv,
 * materialIndex = triangle index) and `materials` (one per triangle); each may be NULL. */
phe_status phe_scene_generate(const phe_scene_recipe* recipe, float* triVerts, phe_triangle_data* datas,
                              phe_material* materials);

/* Host BVH in the reference layout, produced by the project's SBVH builder. */
typedef struct phe_host_bvh phe_host_bvh;
typedef struct phe_sbvh_params {
	float splitAlpha;        /* spatial-split overlap threshold relative to the root area (1e-5) */
	int32_t maxDepth;        /* leaf depth limit (64) */
	int32_t maxSpatialDepth; /* no spatial splits at or below this depth (48) */
	int32_t numThreads;      /* 0 = all hardware threads */
} phe_sbvh_params;
/* Defaults of the reference builder (sbvh-stuff/BVH.h:68-81, SplitBVHBuilder.h:38-44). */
void phe_sbvh_default_params(phe_sbvh_params* params);
/* Spatial-split SAH builder (Stich, Friedrich, Dietrich 2009) over `numTris` triangles given as 9
 * floats each. Output is sanitized like sanitizeBVH (StaticBVHBuilder.cpp:19-78, 253-260): node 0
 * is the root, nodes in depth-first order, leaf indices negated, end markers in .w. Replaces
 * buildStaticFrom (StaticBVHBuilder.cpp:213-251). */
phe_status phe_sbvh_build(const float* triVerts, uint32_t numTris, const phe_sbvh_params* params,
                          phe_host_bvh** out);
phe_status phe_host_bvh_info(const phe_host_bvh* bvh, uint32_t* numNodes, uint32_t* numSlots, uint32_t* maxDepth);
/* Copies nodes, slot vertices and the slot -> input-triangle map (any may be NULL). */
phe_status phe_host_bvh_copy(const phe_host_bvh* bvh, phe_bvh_node* nodes, phe_triangle_vertices* verts,
                             uint32_t* slotToTri);
void phe_host_bvh_free(phe_host_bvh* bvh);

/* Checks a BVH in the reference layout: every node reachable from the root exactly once, child
 * and slot indices in range, leaf counts > 0, leaf depth <= 64. Returns PHE_OK or
 * PHE_ERR_INVALID_SCENE; `maxDepth` (optional) receives the deepest leaf level. */
phe_status phe_bvh_validate(const phe_bvh_node* nodes, uint32_t numNodes, uint32_t numSlots, uint32_t* maxDepth);

/* The 8-wide compressed node layout (PHE_LAYOUT_WIDE8) that scene upload builds from a tree, on the
 * host: 20 words per node and 8 words per leaf record (format in csrc/host/wide8.hpp). Either output
 * array may be NULL to query the counts first. PHE_ERR_INVALID_SCENE (reason in phe_last_error) when the
 * tree allows no 8-wide layout: a child box outside its parent's box, inverted or not finite. No
 * reference counterpart (the reference traverses its binary nodes only). */
phe_status phe_bvh_wide8_build(const phe_bvh_node* nodes, uint32_t numNodes, uint32_t numSlots, uint32_t* nodeWords,
                               uint32_t maxNodes, uint32_t* leafWords, uint32_t maxLeaves, uint32_t* numNodes8,
                               uint32_t* numLeaves8, uint32_t* depth);

/* BVH cache file (testbed_application/Main.cpp:105-154): three headerless raw arrays
 * <base>_nodes.bin, <base>_verts.bin, <base>_datas.bin. Read sizes come from the file sizes;
 * datas must have as many entries as verts (the reference's only check, Main.cpp:131-133). Writes
 * also put <base>_header.bin beside them (magic, version, record sizes, counts, a 64-bit checksum of
 * each array); a read verifies it when it exists (PHE_ERR_INVALID_SCENE on a mismatch) and reads
 * caches without one, as the reference writes them, unchecked. */
phe_status phe_bvh_cache_write(const char* basePath, const phe_bvh_node* nodes, uint32_t numNodes,
                               const phe_triangle_vertices* verts, const phe_triangle_data* datas, uint32_t numSlots);
phe_status phe_bvh_cache_sizes(const char* basePath, uint32_t* numNodes, uint32_t* numSlots);
phe_status phe_bvh_cache_read(const char* basePath, phe_bvh_node* nodes, uint32_t numNodes,
                              phe_triangle_vertices* verts, phe_triangle_data* datas, uint32_t numSlots);

/* generateCameraDef (ray_tracer_common/GenerateRays.cpp:12-35). */
void phe_generate_camera_def(const float pos[3], const float dir[3], const float up[3], float vertFovRad,
                             float resX, float resY, phe_camera_def* out);
/* Entry i (mod 16) of the Halton(2,3) jitter table minus 0.5 (screens/GameScreen.cpp:21-39). */
void phe_halton_jitter(uint32_t index, float out[2]);

/* ---------------------------------------------------------------------------------------------
 * Device scenes
 * ------------------------------------------------------------------------------------------- */

typedef struct phe_scene phe_scene;
#define PHE_PTR_HOST 0
#define PHE_PTR_DEVICE 1
/* Validates and uploads a scene (setStaticScene, CudaTracerRenderer.cpp:251-315): the reference
 * node and triangle arrays are re-laid out on the device into the traversal layout. `datas` and
 * `materials` may be NULL (ray queries only). `where` says whether the array pointers are host
 * or device memory. Synchronous. */
phe_status phe_scene_create(const phe_bvh_node* nodes, uint32_t numNodes, const phe_triangle_vertices* verts,
                            const phe_triangle_data* datas, uint32_t numSlots, const phe_material* materials,
                            uint32_t numMaterials, int where, phe_scene** out);
/* setMaterialsAndTextures (CudaTracerRenderer.cpp:192-239): replaces the scene's materials and
 * textures (host arrays). Every materialIndex of the scene's triangle data must be < numMaterials, every
 * texture index -1 or < numTextures, and albedo textures must have 4 bytes per pixel. Sampling follows
 * the reference's texture objects (CudaBindlessTexture.cpp:66-72: normalized coordinates, wrap, nearest
 * texel): texel i = floor(frac(u) * width) (i = width wraps to 0; NaN -> 0), j likewise with v and height;
 * albedo rgb = powf(byte / 255, 2.2) (InterpretRayHitKernel.cu:41-47) from a table of the correctly
 * rounded values, alpha = byte / 255; roughness and metallic = first byte / 255. Synchronous: waits for
 * the device to finish work that may still read the old arrays. */
phe_status phe_scene_set_materials_and_textures(phe_scene* scene, const phe_material* materials, uint32_t numMaterials,
                                                const phe_texture* textures, uint32_t numTextures);
phe_status phe_scene_destroy(phe_scene* scene);
/* Device bytes held by the scene. */
phe_status phe_scene_device_bytes(const phe_scene* scene, uint64_t* bytes);

/* ---------------------------------------------------------------------------------------------
 * Ray casting (the hot path). Rays and results are device arrays of n entries. The persistent
 * launches (phe_cast_closest, phe_cast_any, batches) take at most PHE_MAX_PERSISTENT_RAYS rays
 * (PHE_ERR_TOO_LARGE above it).
 * ------------------------------------------------------------------------------------------- */
#define PHE_MAX_PERSISTENT_RAYS 0xFC000000u

/* Closest hit, persistent warps with dynamic ray fetch (replaces launchRayCastKernel,
 * RayCastKernel.cu:806-839). */
phe_status phe_cast_closest(const phe_scene* scene, const phe_ray_in* rays, phe_ray_hit* hits, uint32_t n,
                            void* stream);
/* Closest hit, one ray per thread (replaces launchRayCastNoPersistenceKernel, RayCastKernel.cu:841-851). */
phe_status phe_cast_closest_plain(const phe_scene* scene, const phe_ray_in* rays, phe_ray_hit* hits, uint32_t n,
                                  void* stream);
/* Any hit: inLight[i] = 1 when no triangle has tMin <= t < tMax, else 0 (replaces
 * launchShadowRayCastKernel, RayCastKernel.cu:853-886; bool is one byte there too).
 * `scatter` (optional, device) redirects result i to inLight[scatter[i]]. */
phe_status phe_cast_any(const phe_scene* scene, const phe_ray_in* rays, uint8_t* inLight, uint32_t n,
                        const uint32_t* scatter, void* stream);

/* Primary rays (genPrimaryRaysKernel, RayCastKernel.cu:899-919) with a sub-pixel offset
 * (jitterX, jitterY) added to the pixel location; order 0 = row-major, 1 = 8x8-tile-major
 * (getRayIdx, CudaDeviceHelpers.cuh:49-62; needs resX and resY multiples of 8). */
phe_status phe_gen_primary_rays(phe_ray_in* rays, const phe_camera_def* cam, uint32_t resX, uint32_t resY,
                                float jitterX, float jitterY, int order, void* stream);

/* Node layout used by every kernel on this scene. PHE_LAYOUT_BINARY (default): the reference's 2-wide
 * nodes. PHE_LAYOUT_WIDE4: the same tree collapsed to 4-wide 128-byte nodes (child bounds in SoA
 * float4s), built at upload when every grandchild box lies inside its parent box; it visits exactly
 * the leaves the binary traversal visits (the rounded slab test is monotone in the bounds), so results
 * are the same, and it is faster for small coherent launches, slower for large incoherent ones.
 * Rays with a non-finite 1/dir always use the binary nodes. Kernels read the layout when launched. */
#define PHE_LAYOUT_BINARY 0
#define PHE_LAYOUT_WIDE4 1
/* PHE_LAYOUT_WIDE8: the tree collapsed to nodes of up to 8 children whose boxes are stored as 8-bit
 * offsets on a per-node power-of-two grid rounded outward (80 bytes per node, after Ylitie, Karras and
 * Laine, HPG 2017), with one 32-byte record per leaf holding its exact box and slot range. Child
 * boxes are tested with directed rounding (entry distance down, exit up), so a quantized box passes
 * whenever the exact one does; a leaf's exact box is re-tested with the reference arithmetic before
 * its triangles, so the same leaves are intersected as with the binary nodes and results are the
 * same. Built at upload when every child box lies inside its parent box and no box is inverted. */
#define PHE_LAYOUT_WIDE8 2
phe_status phe_scene_set_layout(phe_scene* scene, int layout);
/* `wideAvailable` (optional) receives a mask of the wide layouts the tree allows: 1 = 4-wide, 2 = 8-wide. */
phe_status phe_scene_get_layout(const phe_scene* scene, int* layout, int* wideAvailable);

/* OR of error bits raised by kernels on this scene: single casts, frames, batches, no-alloc batches
 * and serving waves (1 = traversal stack overflow, never set for a scene that passed validation;
 * 2 = a node or slot index outside its array, checked build only). Synchronous. */
phe_status phe_scene_status(const phe_scene* scene, uint32_t* bits);

/* ---------------------------------------------------------------------------------------------
 * Batched multi-scene casting (no reference counterpart: the reference launches and synchronises
 * once per batch, RayCastKernel.cu:806-886). Many batches of uneven size over several resident
 * scenes, closest and any hit mixed, run in ONE persistent launch, replayed from a CUDA graph.
 * ------------------------------------------------------------------------------------------- */
#define PHE_QUERY_CLOSEST 0
#define PHE_QUERY_ANY 1
#define PHE_BATCH_ORDER_GIVEN 0
#define PHE_BATCH_ORDER_LARGEST_FIRST 1
typedef struct phe_batch phe_batch;
typedef struct phe_batch_item {
	uint32_t scene;          /* index into the scene list given to phe_batch_create */
	uint32_t kind;           /* PHE_QUERY_CLOSEST (out: phe_ray_hit[count]) or PHE_QUERY_ANY (out: uint8_t[count]) */
	uint32_t count;
	uint32_t pad;
	const phe_ray_in* rays;  /* device */
	void* out;               /* device */
} phe_batch_item;
typedef struct phe_batch_params {
	int32_t blockSize;       /* 64, 128 or 256 threads */
	int32_t blocksPerSM;     /* resident blocks per SM (0 = occupancy limit) */
	int32_t order;           /* PHE_BATCH_ORDER_* */
	int32_t useGraph;        /* 1 = replay from a CUDA graph captured on first launch */
	int32_t layout;          /* PHE_LAYOUT_* for every scene of the batch (a wide layout only where the scene has it) */
	int32_t stackShared;     /* traversal-stack entries kept in shared memory: 0 or 16 (the rest: local) */
	int32_t sortWindow;      /* ray-sort granularity: 0 = rays in the given order, else 256..4096 (a
	                          * multiple of 256): within windows of that many rays of a batch, rays are
	                          * traced grouped by direction octant (stable); results land at the rays'
	                          * own indices either way */
	int32_t pad;
} phe_batch_params;
typedef struct phe_batch_tuning_row { phe_batch_params params; float ms; } phe_batch_tuning_row;
void phe_batch_default_params(phe_batch_params* params);
/* The batch keeps the scene handles and the item table (device buffers stay owned by the caller).
 * Every scene must live on the current device (PHE_ERR_INVALID_ARGUMENT otherwise). Traversal errors
 * of a launch are ORed into each item's scene status word (phe_scene_status). */
phe_status phe_batch_create(const phe_scene* const* scenes, uint32_t numScenes, const phe_batch_item* items,
                            uint32_t numItems, const phe_batch_params* params, phe_batch** out);
/* New buffers / counts for the same number of items (the captured graph is rebuilt on next launch).
 * update and set_params rewrite the batch's device tables in place: they first wait on the host for the
 * batch's last launch, on whichever stream it ran, and return with the new tables on the device, so the
 * next launch on any stream reads them. */
phe_status phe_batch_update(phe_batch* batch, const phe_batch_item* items, uint32_t numItems);
phe_status phe_batch_set_params(phe_batch* batch, const phe_batch_params* params);
/* One persistent launch over every item, asynchronous on `stream`. */
phe_status phe_batch_launch(phe_batch* batch, void* stream);
phe_status phe_batch_info(const phe_batch* batch, uint64_t* totalRays, uint32_t* paddedRays);
/* Times every candidate (block size x batch order x occupancy x node layout x shared stack depth x ray-sort
 * granularity) `repeats` times on this batch with
 * CUDA events on `stream`, sets the fastest on the batch and returns it; `rows` (optional) receives
 * every candidate's time. Synchronous. */
phe_status phe_batch_autotune(phe_batch* batch, int repeats, void* stream, phe_batch_params* best, float* bestMs,
                              phe_batch_tuning_row* rows, uint32_t maxRows, uint32_t* numRows);
phe_status phe_batch_destroy(phe_batch* batch);
/* The batched launch without any device allocation (no counterpart in the reference). For callers
 * that manage all device memory themselves and cannot let a library call cudaMalloc (an engine's
 * renderer or a plugin host with its own allocator and memory budget; cudaMalloc may also wait for
 * the whole device). The descriptor table, scene table and work counter live in a fixed 12,544-byte
 * array inside the library (per GPU, until exit) instead of device memory the call allocates.
 * At most 256 batch items and 32 scenes per call (PHE_ERR_TOO_LARGE beyond); every scene must live
 * on the current device (PHE_ERR_INVALID_ARGUMENT). All calls share the array: calls whose GPU work
 * overlaps race, so serialise them on one stream. The first call on a device looks up the array's
 * address on that (current) device; make it before any stream capture. The tables travel to the
 * GPU as a kernel parameter (no host-to-device copy), so the call queues two kernels on `stream`
 * and returns without waiting for the GPU; results as phe_batch_launch. Traversal errors are ORed
 * into each item's scene status word: read them with phe_scene_status. */
phe_status phe_batch_cast_noalloc(const phe_scene* const* scenes, uint32_t numScenes, const phe_batch_item* items,
                                  uint32_t numItems, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Wavefront renderer (CudaTracerRenderer, cuda_ray_tracer/CudaTracerRenderer.hpp:14-58, and the
 * BaseRenderer entry points, phantasy_engine/rendering/BaseRenderer.hpp:56-90)
 *
 * One render() is a frame: primary closest hit -> shading + one shadow ray per light -> one
 * bounce ray per hit -> closest hit -> shading + shadow rays -> resolve -> TAA. Shadow and bounce
 * rays are compacted into queues. Colours are linear float RGBA, row-major from the bottom row.
 * ------------------------------------------------------------------------------------------- */
typedef struct phe_renderer phe_renderer;
typedef struct phe_render_result {
	uint32_t resX, resY;
	const float* color;      /* device, float4 per pixel: TAA output (RenderResult::colorTexture) */
	const float* history;    /* device, float4 per pixel: TAA history, alpha = sample count */
	const float* rawColor;   /* device, float4 per pixel: resolved frame before TAA */
	const float* roughness;  /* device, float per pixel: roughness at the primary hit (materialTexture) */
	const float* velocity;   /* device, float2 per pixel: TAA uv velocity of the last frame, NULL when the
	                          * camera stood still (0 everywhere). The reference's velocityTexture holds
	                          * object world velocity, 0 for the static scene; this is what its
	                          * velocity_gen.frag derives from it and the depth buffer. */
} phe_render_result;
phe_status phe_renderer_create(phe_renderer** out);
phe_status phe_renderer_destroy(phe_renderer* renderer);
/* setStaticScene: the scene must carry triangle data and materials. */
phe_status phe_renderer_set_static_scene(phe_renderer* renderer, const phe_scene* scene);
/* setTargetResolution: multiples of 8 (CudaTracerRenderer.cpp:470-471). When the buffers are too small,
 * it reallocates them: it waits for all device work first, and returns with the new buffers cleared, so
 * the next frame on any stream finds them zeroed. */
phe_status phe_renderer_set_target_resolution(phe_renderer* renderer, uint32_t resX, uint32_t resY);
/* updateCamera(ViewFrustum): position, direction, up, vertical FOV in degrees and the TAA pixel
 * offset (ViewFrustum::setPixelOffset, GameScreen.cpp:187-203). */
phe_status phe_renderer_update_camera(phe_renderer* renderer, const float pos[3], const float dir[3], const float up[3],
                                      float vertFovDeg, float pixelOffsetX, float pixelOffsetY);
/* The same with an explicit CameraDef and eye position. */
phe_status phe_renderer_set_camera_def(phe_renderer* renderer, const phe_camera_def* cam, const float camPos[3],
                                       float pixelOffsetX, float pixelOffsetY);
/* Seed of the random streams and the index of the next frame (advanced by each render). */
phe_status phe_renderer_set_seed(phe_renderer* renderer, uint64_t seed, uint32_t frame);
/* 1 = replay the frame from a CUDA graph captured on first use (default 0). */
phe_status phe_renderer_set_graph(phe_renderer* renderer, int enable);
/* Clears the TAA history (GameScreen::resetTAA). */
phe_status phe_renderer_reset_taa(phe_renderer* renderer, void* stream);
/* render(objects, lights): asynchronous on `stream`; lights are host memory (at most 8). */
phe_status phe_renderer_render(phe_renderer* renderer, const phe_sphere_light* lights, uint32_t numLights, void* stream);
phe_status phe_renderer_result(const phe_renderer* renderer, phe_render_result* out);
/* Copies one result buffer to host memory (0 = color, 1 = history, 2 = rawColor: 16 bytes per pixel;
 * 3 = roughness: 4 bytes per pixel; 4 = TAA velocity: 2 floats per pixel, in uv units). Synchronises
 * `stream`. The headless stand-in for reading the GL result texture. */
phe_status phe_renderer_read(const phe_renderer* renderer, int which, void* hostDst, void* stream);
/* Asynchronous read-back for frame pipelines: copies the buffer to `hostDst` on the renderer's copy
 * stream after the work queued on `stream`, overlapping the frames queued after it. Returns at once.
 * Colour, history and velocity are kept per side of the frame parity and copied in place (the frame
 * after next, which rewrites that side, waits for the copy); raw colour and roughness are first
 * snapshot into one of two device staging slots on `stream`. `hostDst` must be pinned for the copy to
 * be asynchronous, and holds the image once phe_renderer_read_wait returns. */
phe_status phe_renderer_read_async(phe_renderer* renderer, int which, void* hostDst, void* stream);
/* Waits until every read_async copy issued so far has landed in host memory. */
phe_status phe_renderer_read_wait(phe_renderer* renderer);
/* Rays cast by the last frame: primary, primary shadow, bounce, bounce shadow. Synchronises `stream`. */
phe_status phe_renderer_ray_counts(const phe_renderer* renderer, uint64_t counts[4], void* stream);

/* Frame pipeline: fused = 1 (the default) runs traversal and shading in one kernel per bounce (6
 * kernels: primary, primary shadow, bounce binning, bounce, bounce shadow, resolve + TAA); 0 splits
 * them (8 kernels: primary trace, primary shade, primary shadow, bounce binning, bounce trace, bounce
 * shade, bounce shadow, resolve + TAA) so the persistent traversal kernels refill idle lanes with new
 * rays when fewer than `refill` (0..32, default 28) lanes of a warp are still busy. sortWindow (0 or
 * a multiple of 256 up to 4096; default 0) bins the bounce rays by direction octant within windows of
 * that many queue entries before they are traced. */
phe_status phe_renderer_set_pipeline(phe_renderer* renderer, int fused, int refill, int sortWindow);
/* Schedule of the two shadow (any-hit) passes of the fused pipeline; every schedule gives the same
 * bytes. IN_ORDER: primary shadows after the primary pass, bounce shadows after the bounce pass.
 * BESIDE_BOUNCE: the primary shadow pass on a second stream of the renderer beside the bounce pass
 * (two parallel graph branches). MERGED (default): one any-hit pass over both queues after the bounce
 * pass, bounce shadows first, so that the short bounce-shadow queue is not a launch of its own that
 * is mostly tail. Frames timed per kernel run BESIDE_BOUNCE in order. */
#define PHE_SHADOWS_IN_ORDER 0
#define PHE_SHADOWS_BESIDE_BOUNCE 1
#define PHE_SHADOWS_MERGED 2
phe_status phe_renderer_set_shadow_schedule(phe_renderer* renderer, int schedule);
/* Per-kernel timing with CUDA events on the render stream (direct launches; ignored while a graph is
 * replayed). Enabling resets the totals. kernel_times returns the summed milliseconds per frame kernel
 * (in launch order, `numKernels` of them) and the number of frames timed. */
phe_status phe_renderer_set_kernel_timing(phe_renderer* renderer, int enable);
/* Bytes copied host -> device per frame (the frame parameter block: camera, jitter, lights). */
uint32_t phe_renderer_frame_param_bytes(void);
phe_status phe_renderer_kernel_times(phe_renderer* renderer, double msTotal[8], uint32_t* numKernels, uint32_t* frames);
/* Frames in flight (no reference counterpart; the reference renders and presents one frame at a time).
 * 1 (default): a frame's kernels run on the stream given to phe_renderer_render. 2: frame k's traversal
 * kernels run on the renderer's traversal stream k % 2 with per-frame buffers of their own, after the
 * work enqueued on the caller's stream before the call and after the resolve that last used those
 * buffers; its resolve + TAA runs on the renderer's resolve stream after the previous frame's resolve.
 * Consecutive frames overlap on the GPU; every frame gives exactly the bytes it gives with 1. The
 * caller's stream is NOT ordered after the frame: phe_renderer_read / read_async / ray_counts /
 * reset_taa / the ray-total calls wait for the last frame themselves, phe_renderer_join orders a stream
 * after it (needed before using the pointers of phe_renderer_result on the GPU). Frames in flight are
 * launched directly (no graph replay); frames timed per kernel run in order on the caller's stream, and
 * the BESIDE_BOUNCE shadow schedule runs IN_ORDER. phe_scene_destroy waits for all device work.
 * Changing the setting waits for the frames in flight; 2 adds a second set of per-frame buffers
 * (~410 MB at 1080p with one light). If making them fails, the call returns the error and frames stay
 * one at a time. */
phe_status phe_renderer_set_frames_in_flight(phe_renderer* renderer, int frames);
/* Split frames (no reference counterpart). 1 (default): a frame's kernels run as one sequence. 2..4:
 * the frame's tile rows (8-pixel rows) are dealt round-robin to `parts` parts, part 0 on the caller's
 * stream and the others on the renderer's part streams forked from it, each with its own ray queues and
 * counters over the shared per-pixel buffers, and the caller's stream joins them at the end of the frame:
 * the stream semantics of one frame are unchanged and every pixel gets the bytes of the whole frame (each
 * pixel's work depends only on the pixel; TAA reads only the previous frame). The parts' kernels overlap
 * on the GPU. Applies to the fused pipeline (at most one part per tile row), not to frames timed per
 * kernel; cannot be combined with two frames in flight; each part past the first adds a set of ray queues.
 * If making them fails, the call returns the error and the previous setting stays. */
phe_status phe_renderer_set_frame_parts(phe_renderer* renderer, int parts);
phe_status phe_renderer_join(phe_renderer* renderer, void* stream);
/* With 2 frames in flight and recording enabled, each frame's GPU latency (start of its first kernel to
 * the end of its resolve) is recorded. frame_latencies with capacity 0 returns how many are recorded;
 * otherwise it waits for and removes up to `capacity` of them, oldest first, into ms[]. */
phe_status phe_renderer_set_latency_recording(phe_renderer* renderer, int enable);
phe_status phe_renderer_frame_latencies(phe_renderer* renderer, float* ms, uint32_t capacity, uint32_t* count);

/* Ray totals per pass summed over the frames since the last reset (device counters): reset clears them
 * on `stream`; totals_async copies the 4 totals (primary, primary shadow, bounce, bounce shadow) to
 * host memory on `stream` (pinned memory for a truly asynchronous copy). */
phe_status phe_renderer_reset_ray_totals(phe_renderer* renderer, void* stream);
phe_status phe_renderer_ray_totals_async(const phe_renderer* renderer, uint64_t* hostTotals4, void* stream);

/* Display post-process for image dumps (gamma_correction.frag:20-74: Uncharted 2 tonemap, then
 * pow(rgb, 1/gamma)) of a linear float4 image into `display` (float4) and/or `rgba8` (4 bytes per
 * pixel, rounded from [0, 1]); either output may be NULL. */
phe_status phe_postprocess(uint32_t resX, uint32_t resY, const float* linear, float gamma, float* display, uint8_t* rgba8,
                           void* stream);
/* Display scaling pass (resources/shaders/scaling.frag:19-35, drawn by GameScreen.cpp:268-273): resamples
 * the rendered region (the first viewportW x viewportH texels of a srcW x srcH float4 image) to dstW x dstH.
 * Each destination pixel averages four GL_LINEAR, clamp-to-edge taps at +-1/4 destination pixel around
 * its centre (uv = (x + 0.5) / dstW, (y + 0.5) / dstH; coord = uv * viewport / src); alpha = 1. Writes
 * float4 `dst` and/or 8-bit RGBA `dstRgba8` (either may be NULL). Asynchronous on `stream`. */
phe_status phe_scale(uint32_t srcW, uint32_t srcH, const float* src, uint32_t viewportW, uint32_t viewportH,
                     uint32_t dstW, uint32_t dstH, float* dst, uint8_t* dstRgba8, void* stream);

/* TAA resolve alone (taa.frag:25-71) on device float4 buffers; velocity and prevVelocity are float2
 * uv velocities (NULL = static), roughness float (NULL = 0). */
phe_status phe_taa_resolve(uint32_t resX, uint32_t resY, const float* cur, const float* hist, const float* velocity,
                           const float* prevVelocity, const float* roughness, float* outColor, float* outHist,
                           void* stream);

/* ---------------------------------------------------------------------------------------------
 * Serving (no reference counterpart): continuous batching of ray-query and render requests against
 * device-resident scenes. A scheduler thread admits requests in arrival order while they fit the
 * device-memory budget (resident scenes count against it), the in-flight limit and, for renders, a
 * free render slot. A render waiting for a slot does not hold back the ray queries behind it; when a
 * slot frees, a render on a scene that another slot is rendering may go before up to 16 earlier
 * pending entries (a render is passed over at most 8 times). Admitted ray queries whose rays are on
 * the device join the next wave, ONE batched
 * persistent launch over all of them; requests arriving meanwhile join the following wave. Renders
 * run their spp frames (wavefront frame + TAA with Halton jitter) on their slot's own stream, so they
 * overlap each other and the query waves. Results go straight to the caller's host buffers (pinned
 * memory gives truly asynchronous copies). `serial` = 1 is the baseline: one request at a time, plain
 * per-request launches, each waited for.
 * ------------------------------------------------------------------------------------------- */
#define PHE_REQ_CLOSEST 0
#define PHE_REQ_ANY 1
#define PHE_REQ_RENDER 2
typedef struct phe_server phe_server;
typedef struct phe_server_config {
	uint64_t memoryBudget;     /* device bytes scenes + in-flight requests may hold (default 120 GiB) */
	uint32_t maxInFlight;      /* admitted requests at once (default 256) */
	uint32_t renderSlots;      /* concurrent renders, each with its own frame buffers (default 4) */
	uint32_t maxRenderPixels;  /* largest render (default 1920*1080; width <= 1920) */
	uint32_t maxLights;        /* lights per render (default 4, at most 8) */
	int32_t serial;            /* 1 = serial baseline */
	uint32_t batchWindowUs;    /* a wave waits up to this long after its first query was admitted to
	                              gather more (0 = launch as soon as a wave slot is free) */
} phe_server_config;
typedef struct phe_request {
	uint32_t kind;             /* PHE_REQ_* */
	uint32_t scene;            /* id from phe_server_add_scene */
	uint32_t numRays;          /* queries */
	uint32_t spp;              /* renders: frames accumulated through TAA */
	const phe_ray_in* rays;    /* queries: host rays */
	void* out;                 /* host: phe_ray_hit[numRays] (closest), uint8_t[numRays] (any), float4[resX*resY] (render) */
	uint32_t resX, resY;       /* renders: multiples of 8 */
	uint32_t numLights, pad;
	phe_camera_def cam;
	float camPos[3];
	float pad2;
	const phe_sphere_light* lights; /* host, copied at submit */
	uint64_t seed;
} phe_request;
typedef struct phe_request_stats {
	double submitMs, admitMs, doneMs; /* milliseconds since the server was created */
	uint64_t rays;                    /* rays cast for the request */
	phe_status status;
	uint32_t pad;
} phe_request_stats;
typedef struct phe_server_stats {
	uint64_t waves, raysCompleted, bytesInUse;
	uint32_t pending, inFlight;
} phe_server_stats;
void phe_server_default_config(phe_server_config* config);
phe_status phe_server_create(const phe_server_config* config, phe_server** out);
/* Registers a resident scene (the server does not own it); returns its id. */
phe_status phe_server_add_scene(phe_server* server, const phe_scene* scene, uint32_t* sceneId);
/* Queues a request (never blocks on the GPU). PHE_ERR_BUDGET if it alone cannot fit the budget. */
phe_status phe_server_submit(phe_server* server, const phe_request* request, uint64_t* requestId);
/* PHE_OK with stats when done, PHE_ERR_NOT_READY while running. */
phe_status phe_server_poll(phe_server* server, uint64_t requestId, phe_request_stats* stats);
phe_status phe_server_wait(phe_server* server, uint64_t requestId, phe_request_stats* stats);
phe_status phe_server_drain(phe_server* server);
/* Forgets a completed request. */
phe_status phe_server_release(phe_server* server, uint64_t requestId);
/* Cancels a request that has not been admitted yet: it completes at once with status
 * PHE_ERR_CANCELLED and its output buffer is never written. An admitted request cannot be cancelled
 * (its work is on the GPU): PHE_ERR_NOT_READY, and it completes normally. */
phe_status phe_server_cancel(phe_server* server, uint64_t requestId);
phe_status phe_server_get_stats(phe_server* server, phe_server_stats* stats);
phe_status phe_server_destroy(phe_server* server);

#ifdef __cplusplus
}
#endif
#endif /* PHE_GB300_H */
