/* Test infrastructure only (the oracle). A plain-C restatement of the reference's CPU ray-cast
 * path, its any-hit semantics, primary-ray generation, wavefront shading, diffuse bounce and TAA
 * resolve. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and reference legs may
 * load it; the product never does.
 *
 * Parity pin: oracle_cast_rays() in reference mode is checked bit-for-bit against the reference's
 * own castRay (compiled from its sources into oracle/_ref/libpheref.so) and against the committed
 * fixtures in tests/golden/ that the reference produced; the shading, sampling and hit-interpretation
 * functions are checked against the reference's own ones compiled as host code
 * (oracle/_ref/libpheref_shading.so) to within 1e-4 absolute, and against their committed outputs.
 *
 * Paths below are relative to the reference project root. Every float operation is written in the
 * reference's source order and the library is built without FP contraction or fast-math, so results
 * are identical on x86-64 and aarch64. */
#ifndef PHE_ORACLE_H
#define PHE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* BVHNode (ray_tracer_common/BVHNode.hpp:23-149), 64 bytes. */
typedef struct { float f[12]; int32_t i[4]; } or_node;
/* TriangleVertices (ray_tracer_common/Triangle.hpp:17-23), 48 bytes. */
typedef struct { float v0[4], v1[4], v2[4]; } or_tri;
/* TriangleData (ray_tracer_common/Triangle.hpp:25-37), 64 bytes. */
typedef struct { float n0[3], n1[3], n2[3], uv0[2], uv1[2], uv2[2]; uint32_t materialIndex; } or_tri_data;
/* RayIn (cuda_ray_tracer/kernels/RayCastKernel.hpp:22-37), 32 bytes: origin, tMin, dir, tMax. */
typedef struct { float o[3]; float tmin; float d[3]; float tmax; } or_ray;
/* RayHit (cuda_ray_tracer/kernels/RayCastKernel.hpp:39-45), 16 bytes. */
typedef struct { uint32_t tri; float t, u, v; } or_hit;
/* CameraDef (ray_tracer_common/GenerateRays.hpp:14-24). */
typedef struct { float origin[3], dir[3], dX[3], dY[3]; } or_camera;
/* SphereLight (level/SphereLight.hpp:13-26) as used by the shading code. */
typedef struct { float pos[3]; float radius; float range; float strength[3]; int32_t staticShadows; } or_light;
/* Material (rendering/Material.hpp:17-55): texture indices (albedo, roughness, metallic, unused;
 * -1 = none), albedo rgba, roughness, metallic, two unused floats. */
typedef struct { int32_t texIndex[4]; float albedo[4]; float roughness; float metallic; float pad[2]; } or_material;
/* Texture (RawImage, rendering/RawImage.hpp:21-28): 8-bit channels, rows `pitch` bytes apart. */
typedef struct { const uint8_t* data; int32_t width, height; uint32_t bytesPerPixel, pitch; } or_texture;

/* Semantics of the accept rule.
 * OR_MODE_REFERENCE_CPU: castRay (BVHTraversal.hpp:37-128): accept t < closest && tMin <= t <= tMax.
 * OR_MODE_REFERENCE_GPU: rayCastKernel (RayCastKernel.cu:361): accept tMin <= t < current, where
 *   current starts at min(tMax, FLT_MAX); a miss reports t = tMax, u = v = 0. */
enum { OR_MODE_REFERENCE_CPU = 0, OR_MODE_REFERENCE_GPU = 1 };

/* Intersection.hpp:24-67 (Moller-Trumbore, absolute |a| < 1e-5 reject). Returns 1 on hit. */
int oracle_intersect_tri(const or_tri* tri, const float o[3], const float d[3], float* t, float* u, float* v);

/* One closest-hit query (BVHTraversal.hpp:37-128 / castDebugRay :223-327). Returns 0, or -1 when
 * the 144-entry stack would overflow (the reference does not check; valid SBVHs never do). */
int oracle_cast_ray(const or_node* nodes, const or_tri* tris, const or_ray* ray, int mode, or_hit* out,
                    uint32_t* nodesVisited, uint32_t* triTests);

/* Batch closest hit over `n` rays with `threads` pthreads (dynamic 64-ray chunks). `debug` is
 * optional: 2 uint32 per ray (nodesVisited, triangleIntersectionTests). Returns the number of
 * rays whose stack would overflow (0 for valid input). */
int oracle_cast_rays(const or_node* nodes, const or_tri* tris, const or_ray* rays, uint32_t n, int mode,
                     or_hit* hits, uint32_t* debug, int threads);

/* Any-hit: inLight[i] = 1 when no triangle has tMin <= t < tMax (shadowRayCastKernel,
 * RayCastKernel.cu:759-765; the reference has no CPU any-hit, so this is castRay in GPU mode). */
int oracle_any_rays(const or_node* nodes, const or_tri* tris, const or_ray* rays, uint32_t n,
                    uint8_t* inLight, int threads);

/* Brute-force closest hit over `numTris` triangles in array order (CPU accept rule in `mode`). */
void oracle_brute_closest(const or_tri* tris, uint32_t numTris, const or_ray* rays, uint32_t n, int mode,
                          or_hit* hits);

/* generateCameraDef (GenerateRays.cpp:12-35). */
void oracle_camera_def(const float pos[3], const float dir[3], const float up[3], float vfovRad,
                       float resX, float resY, or_camera* out);

/* Index of pixel (x, y) in the ray buffer: order 0 = row-major (CPUTracerRenderer.cpp:84-99),
 * order 1 = 8x8-tile-major (getRayIdx, CudaDeviceHelpers.cuh:49-62). */
uint32_t oracle_ray_index(uint32_t x, uint32_t y, uint32_t resX, int order);

/* Primary rays (genPrimaryRaysKernel RayCastKernel.cu:891-919) with a sub-pixel offset
 * (jx, jy) added to the pixel location (GameScreen.cpp:187-203): tMin 1e-4, tMax FLT_MAX. */
void oracle_gen_primary(const or_camera* cam, uint32_t resX, uint32_t resY, float jx, float jy, int order,
                        or_ray* rays);

/* PCG32 (O'Neill 2014, XSH-RR 64/32), the random stream shared by the GPU and the oracle. */
typedef struct { uint64_t state, inc; } or_pcg;
void oracle_pcg_seed(or_pcg* r, uint64_t initstate, uint64_t initseq);
uint32_t oracle_pcg_next(or_pcg* r);
float oracle_pcg_uniform(or_pcg* r);
/* Seed of the stream of pixel `pixel` for `stage` in `frame`. */
void oracle_pixel_stream(or_pcg* r, uint64_t seed, uint32_t frame, uint32_t pixel, uint32_t stage);
/* sin(2 pi r) and cos(2 pi r) for r in [0, 1): quadrant reduction plus Taylor polynomials, written
 * with single roundings so the GPU reproduces it bit for bit. */
void oracle_sincos_2pi(float r, float* s, float* c);

/* shade() / falloffFactor() (CudaPbr.cuh:26-111). Integer powers are repeated products. */
void oracle_shade(const float p[3], const float n[3], const float v[3], const float albedo[3], float roughness,
                  float metallic, const float l[3], float toLightDist, const float strength[3], float range,
                  float out[3]);
float oracle_falloff(float toLightDist, float range);

/* Cosine-weighted bounce direction (sampleLambertian + hemisphereToWorld, MaterialKernel.cu:206-246). */
void oracle_sample_lambert(float r1, float r2, const float n[3], float out[3]);
/* The GGX branch of the bounce (createSecondaryRaysKernel, MaterialKernel.cu:293-299): sampleGgx with
 * a = roughness^2 around reflect(fromCamera, n) (CudaDeviceHelpers.cuh:44-47, MaterialKernel.cu:221-237). */
void oracle_sample_ggx_bounce(float r1, float r2, float roughness, const float fromCamera[3], const float n[3],
                              float out[3]);
/* retrieveTriData (InterpretRayHitKernel.cu:13-37) for n hits, row i reading datas[i]: out receives
 * pos.xyz, normal.xyz, uv.xy (8 floats per row). */
void oracle_retrieve_tri_data(uint32_t n, const or_tri_data* datas, const or_ray* rays, const or_hit* hits, float* out,
                              uint32_t* materialIndex);
/* shadeHit (MaterialKernel.cu:49-112) for one light with the two uniform numbers r12 of its soft-shadow
 * offset: contribution = mask * falloff * shade(...); returns 1 and fills shadowRay when the light
 * casts a shadow ray, 0 where the reference writes its dummy ray. */
int oracle_shade_hit(const or_light* light, const float mask[3], const float normal[3], const float toCamera[3],
                     const float pos[3], const float albedo[3], float metallic, float roughness, const float r12[2],
                     float contrib[3], or_ray* shadowRay);

/* Wavefront frame (CudaTracerRenderer.cpp:612-728 normal path, with the raster G-buffer replaced
 * by ray-cast primary hits): primary closest hit -> shade + one shadow ray per light -> cosine
 * bounce -> closest hit -> shade + shadow rays -> sum of lit contributions. `color` receives
 * resX*resY float4 (rgb, 1) in row-major pixel order; `roughnessOut` (optional) the per-pixel
 * roughness the TAA pass reads. `primaryHits` (optional) supplies the primary closest hits in
 * row-major order instead of casting them (used to check stages in isolation). */
typedef struct {
	uint32_t resX, resY;
	or_camera cam;            /* jittered camera (pixel offset applied in ray generation) */
	float jitter[2];
	float camPos[3];
	const or_light* lights; uint32_t numLights;
	const or_material* materials;
	uint64_t seed; uint32_t frame;
	const or_texture* textures; uint32_t numTextures;
	uint32_t rowBegin, rowEnd;  /* rows rendered: [rowBegin, rowEnd), rowEnd = 0 meaning resY */
	/* Camera motion (velocity_gen.frag with a ray-cast surface): when `velocity` is set, it receives
	 * per pixel (row-major float2) the uv of the primary surface point (or of the ray direction on a
	 * miss) in `cam` minus its uv in `prevCam`, both without jitter; (2, 2) behind either camera. */
	or_camera prevCam;
	float* velocity;
	/* Ray dump (optional): every ray cast at stage s (primary, primary shadow, bounce, bounce shadow) is
	 * also written to dump[s] (up to dumpCapacity[s] rays, in no particular order); dumpCount[s] receives
	 * the number cast. Lets a CPU baseline time another traversal on exactly the frame's rays. */
	or_ray* dump[4];
	uint32_t dumpCapacity[4];
	uint32_t* dumpCount;
} or_frame_params;
/* `rayCounts` (optional, 4): rays cast per stage (primary, primary shadow, bounce, bounce shadow);
 * `workSums` (optional, 8): castDebugRay's nodesVisited and triangleIntersectionTests summed per stage. */
int oracle_render_frame(const or_node* nodes, const or_tri* tris, const or_tri_data* datas,
                        const or_frame_params* fp, const or_hit* primaryHits, float* color, float* roughnessOut,
                        uint64_t* rayCounts, uint64_t* workSums, int threads);

/* Nearest-texel index along one axis for a normalized coordinate with wrap addressing (the
 * reference's texture objects, CudaBindlessTexture.cpp:66-72): floor(frac(c) * n), with n wrapping
 * to 0 and a NaN or infinite coordinate giving 0. */
uint32_t oracle_texel_coord(float c, int32_t n);
/* powf(b / 255, 2.2) (InterpretRayHitKernel.cu:41-47), correctly rounded, for b = 0..255. */
void oracle_srgb_table(float out[256]);

/* TAA resolve (resources/shaders/taa.frag:25-71) on row-major float4 buffers. velocity and
 * prevVelocity are float2 uv-velocities (NULL = zero). History alpha holds the sample count. */
void oracle_taa(uint32_t resX, uint32_t resY, const float* cur, const float* hist, const float* velocity,
                const float* prevVelocity, const float* roughness, float* outColor, float* outHist);

/* Display post-process (gamma_correction.frag:20-74): Uncharted 2 tonemap then pow(rgb, 1/gamma), on
 * n float4 pixels; alpha passes through. */
/* Display scaling pass (scaling.frag:19-35): the viewport part of a float4 source resampled to the
 * destination by averaging four GL_LINEAR clamp-to-edge taps at +-1/4 destination pixel. */
void oracle_scale(uint32_t srcW, uint32_t srcH, const float* src, uint32_t vpW, uint32_t vpH, uint32_t dstW,
                  uint32_t dstH, float* dst);
void oracle_postprocess(uint32_t n, const float* linear, float gamma, float* display);

/* Halton(2,3) jitter table entry i - 0.5 (GameScreen.cpp:21-39). */
void oracle_halton_jitter(uint32_t i, float out[2]);

#ifdef __cplusplus
}
#endif
#endif
