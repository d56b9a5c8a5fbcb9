// Test infrastructure only: the reference's own shading, sampling and hit-interpretation functions
// compiled as host code, behind an extern "C" batch interface, so that the oracle's restatement of
// them (oracle/oracle.c) can be checked against the reference itself. Built by oracle/Makefile into
// oracle/_ref/libpheref_shading.so (git-ignored); nothing in the product links it.
//
// Reference functions (paths relative to the reference project root):
//   ggx / geometricSchlick / fresnelSchlick / shade / falloffFactor
//                                 source/cuda_ray_tracer/CudaPbr.cuh:26-111 (header, included as is)
//   lerp / clamp / reflect        source/cuda_ray_tracer/CudaDeviceHelpers.cuh:24-47 (header)
//   setToDummyRay / shadeHit      source/cuda_ray_tracer/kernels/MaterialKernel.cu:41-112
//   hemisphereToWorld / clampToHemisphere / sampleGgx / sampleLambertian
//                                 source/cuda_ray_tracer/kernels/MaterialKernel.cu:206-246
//   retrieveTriData               source/cuda_ray_tracer/kernels/InterpretRayHitKernel.cu:13-37
// The .cu functions are copied out of the reference files at build time by oracle/ref_extract.py
// (the kernels around them need a CUDA compiler; these functions do not).
//
// Host compilation notes: every function is `__device__`, which the CUDA headers turn into an
// attribute the host compiler ignores. CUDA device code calls the float overloads of fma, abs, sqrt,
// cos and sin; the using-declarations below give host code the same float overloads (without them
// unqualified abs(float) could bind to the integer abs). curand_uniform is replaced by a stream of
// numbers given by the caller, so both sides can be fed the same random numbers.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace phe {
using std::abs;
using std::cos;
using std::fma;
using std::isfinite;
using std::sin;
using std::sqrt;
} // namespace phe

#include "cuda_ray_tracer/CudaPbr.cuh"
#include "cuda_ray_tracer/kernels/RayCastKernel.hpp"
#include "phantasy_engine/level/SphereLight.hpp"
#include "phantasy_engine/ray_tracer_common/Triangle.hpp"

// Stand-in for curand's state: the caller's uniform numbers in order.
struct curandState {
	const float* next;
};
static inline float curand_uniform(curandState* s) { return *s->next++; }

namespace phe {
using sfz::vec2;
using sfz::vec2u;
using sfz::vec3;
using sfz::vec4;
#include "ref_extracted.inc"
} // namespace phe

using namespace phe;

static vec3 v3(const float* p) { return vec3(p[0], p[1], p[2]); }
static void put3(float* o, const vec3& v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }

extern "C" {

// shade(): rows of 22 floats p.xyz n.xyz v.xyz albedo.rgb roughness metallic l.xyz toLightDist
// strength.rgb range -> 3 floats.
void ref_shade(uint32_t n, const float* in, float* out)
{
	for (uint32_t i = 0; i < n; i++) {
		const float* r = in + 22 * (size_t)i;
		vec3 s = shade(v3(r), v3(r + 3), v3(r + 6), v3(r + 9), r[12], r[13], v3(r + 14), r[17], v3(r + 18), r[21]);
		put3(out + 3 * (size_t)i, s);
	}
}

void ref_falloff(uint32_t n, const float* dist, const float* range, float* out)
{
	for (uint32_t i = 0; i < n; i++) out[i] = falloffFactor(dist[i], range[i]);
}

// sampleLambertian(): rows r1 r2 n.xyz -> 3 floats.
void ref_sample_lambertian(uint32_t n, const float* in, float* out)
{
	for (uint32_t i = 0; i < n; i++) {
		const float* r = in + 5 * (size_t)i;
		put3(out + 3 * (size_t)i, sampleLambertian(vec2(r[0], r[1]), v3(r + 2)));
	}
}

// sampleGgx() as the secondary-ray kernel calls it (MaterialKernel.cu:296-299): rows r1 r2 roughness
// fromCamera.xyz n.xyz -> 3 floats; a = roughness^2, reflection = reflect(fromCamera, n).
void ref_sample_ggx(uint32_t n, const float* in, float* out)
{
	for (uint32_t i = 0; i < n; i++) {
		const float* r = in + 9 * (size_t)i;
		vec3 nn = v3(r + 6);
		vec3 reflection = reflect(v3(r + 3), nn);
		float a = r[2] * r[2];
		put3(out + 3 * (size_t)i, sampleGgx(vec2(r[0], r[1]), a, reflection, nn));
	}
}

// retrieveTriData(): datas = TriangleData per hit (64 bytes), rays = RayIn, hits = RayHit ->
// pos.xyz normal.xyz uv.xy per row (8 floats) and the material index.
void ref_retrieve_tri_data(uint32_t n, const void* datas, const void* rays, const void* hits, float* out,
                           uint32_t* materialIndex)
{
	const TriangleData* d = (const TriangleData*)datas;
	const RayIn* ry = (const RayIn*)rays;
	const RayHit* h = (const RayHit*)hits;
	for (uint32_t i = 0; i < n; i++) {
		RayHit hit = h[i];
		hit.triangleIndex = i;   // row i reads datas[i]
		vec3 pos, normal;
		vec2 uv;
		uint32_t mi = 0;
		retrieveTriData(d, ry[i], hit, pos, normal, uv, mi);
		float* o = out + 8 * (size_t)i;
		put3(o, pos);
		put3(o + 3, normal);
		o[6] = uv.x;
		o[7] = uv.y;
		materialIndex[i] = mi;
	}
}

// shadeHit() for one light (MaterialKernel.cu:49-112): rows of 28 floats mask.rgb normal.xyz
// toCamera.xyz pos.xyz albedo.rgb metallic roughness light.pos.xyz light.radius light.range
// light.strength.rgb light.staticShadows r1 r2 -> contribution.rgb and the shadow ray (8 floats) per
// row; cast[i] = 0 where the reference writes its dummy ray instead.
void ref_shade_hit(uint32_t n, const float* in, float* contribution, float* shadowRay, uint8_t* cast)
{
	for (uint32_t i = 0; i < n; i++) {
		const float* r = in + 28 * (size_t)i;
		SphereLight light;
		light.pos = v3(r + 17);
		light.radius = r[20];
		light.range = r[21];
		light.strength = v3(r + 22);
		light.staticShadows = r[25] != 0.0f;
		curandState rs{r + 26};
		RayIn ray;
		vec3 contrib;
		shadeHit(0, 1, v3(r), rs, &ray, &contrib, v3(r + 3), v3(r + 6), v3(r + 9), v3(r + 12), r[15], r[16], &light, 1);
		put3(contribution + 3 * (size_t)i, contrib);
		std::memcpy(shadowRay + 8 * (size_t)i, &ray, sizeof(RayIn));
		// setToDummyRay: origin (1e6, 1e6, 1e6), tMin = tMax = 0.001 (MaterialKernel.cu:41-47)
		cast[i] = !(ray.origin().x == 1000000.0f && ray.minDist() == 0.001f && ray.maxDist() == 0.001f);
	}
}

} // extern "C"
