// Device shading: shade() / falloffFactor() (cuda_ray_tracer/CudaPbr.cuh:26-111), the per-light
// part of shadeHit (kernels/MaterialKernel.cu:49-112), hit interpretation (retrieveTriData,
// InterpretRayHitKernel.cu:13-37) and bounce sampling (createSecondaryRaysKernel,
// MaterialKernel.cu:206-312). Integer powers are written as products and the random numbers come
// from PCG32, so the host oracle reproduces every value bit for bit.
#pragma once

#include "common.cuh"

namespace phe_gb300 {

constexpr float kPiF = 3.14159274f;
constexpr double kPiD = 3.141592653589793;

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
// lerp of CudaDeviceHelpers.cuh:24-27.
__device__ __forceinline__ float lerpf(float v0, float v1, float t) { return __fmaf_rn(t, v1, __fmaf_rn(-t, v0, v0)); }

__device__ __forceinline__ float ggx(float nDotH, float a)
{
	float a2 = __fmul_rn(a, a);
	float base = __fadd_rn(__fmul_rn(__fmul_rn(nDotH, nDotH), __fsub_rn(a2, 1.0f)), 1.0f);
	float div = __double2float_rn(__dmul_rn(kPiD, (double)__fmul_rn(base, base)));
	return __fdiv_rn(a2, div);
}

__device__ __forceinline__ float geometric_schlick(float nDotL, float nDotV, float k)
{
	float omk = __fsub_rn(1.0f, k);
	float g1 = __fdiv_rn(nDotL, __fadd_rn(__fmul_rn(nDotL, omk), k));
	float g2 = __fdiv_rn(nDotV, __fadd_rn(__fmul_rn(nDotV, omk), k));
	return __fmul_rn(g1, g2);
}

__device__ __forceinline__ f3 shade(f3 n, f3 v, f3 albedo, float roughness, float metallic, f3 l, float toLightDist,
                                    f3 strength, float range)
{
	f3 zero = mk3(0.0f, 0.0f, 0.0f);
	if (toLightDist > range) return zero;
	f3 h = normalize3(add3(l, v));
	float nDotL = dot3(n, l);
	if (nDotL <= 0.0f) return zero;
	float nDotV = fmaxf(0.001f, dot3(n, v));
	f3 diffuse = divs3(albedo, kPiF);
	float nDotH = fmaxf(0.0f, dot3(n, h));
	float ctD = ggx(nDotH, __fmul_rn(roughness, roughness));
	float rp1 = __fadd_rn(roughness, 1.0f);
	float k = __fdiv_rn(__fmul_rn(rp1, rp1), 8.0f);
	float ctG = geometric_schlick(nDotL, nDotV, k);
	f3 f0 = mk3(lerpf(0.04f, albedo.x, metallic), lerpf(0.04f, albedo.y, metallic), lerpf(0.04f, albedo.z, metallic));
	float om = __fsub_rn(1.0f, nDotV);
	float om2 = __fmul_rn(om, om);
	float p5 = clampf(__fmul_rn(__fmul_rn(om2, om2), om), 0.0f, 1.0f);
	f3 one = mk3(1.0f, 1.0f, 1.0f);
	f3 ctF = add3(f0, muls3(sub3(one, f0), p5));
	f3 specular = divs3(muls3(muls3(ctF, ctD), ctG), __fmul_rn(__fmul_rn(4.0f, nDotL), nDotV));
	f3 kd = muls3(sub3(one, ctF), __fsub_rn(1.0f, metallic));
	f3 shaded = muls3(mul3(add3(mul3(kd, diffuse), specular), strength), nDotL);
	if (!isfinite(shaded.x) || !isfinite(shaded.y) || !isfinite(shaded.z)) shaded = zero;
	return shaded;
}

__device__ __forceinline__ float falloff(float toLightDist, float range)
{
	float x = __fdiv_rn(toLightDist, range);
	float x2 = __fmul_rn(x, x);
	float c = clampf(__fsub_rn(1.0f, __fmul_rn(x2, x2)), 0.0f, 1.0f);
	float num = __fmul_rn(c, c);
	float den = __double2float_rn(__dadd_rn((double)__fmul_rn(toLightDist, toLightDist), 1.0));
	return __fdiv_rn(num, den);
}

struct HitInfo {
	f3 pos, normal;
	f3 albedo;
	float alpha, roughness, metallic;
};

// Nearest texel index along one axis of a normalized, wrapping texture coordinate (the reference's
// texture objects, CudaBindlessTexture.cpp:66-72): floor(frac(c) * n), n wrapping to 0, NaN to 0.
__device__ __forceinline__ uint32_t texel_coord(float c, int32_t n)
{
	float f = __fsub_rn(c, floorf(c));
	if (!(f >= 0.0f)) return 0u;   // NaN or infinite coordinate
	uint32_t i = (uint32_t)__fmul_rn(f, (float)n);
	return i >= (uint32_t)n ? 0u : i;
}

// Address of texel (u, v) of texture `ti` (validated on upload: ti < numTextures).
__device__ __forceinline__ const uint8_t* texel(const DeviceScene& s, int32_t ti, float u, float v)
{
	const DeviceTexture t = s.textures[ti];
	uint32_t i = texel_coord(u, t.width), j = texel_coord(v, t.height);
	return s.texels + t.offset + (uint64_t)j * t.rowBytes + (uint64_t)i * t.bytesPerPixel;
}

// retrieveTriData + the material part of interpretRayHitKernel (InterpretRayHitKernel.cu:13-37,
// 60-121): position, interpolated normal and uv, material constants or texels.
__device__ __forceinline__ HitInfo interpret_hit(const DeviceScene& s, f3 o, f3 d, uint32_t slot, float t, float u,
                                                 float v)
{
	const phe_triangle_data& td = s.datas[slot];
	HitInfo hi;
	hi.pos = add3(o, muls3(d, t));
	f3 n0 = mk3(td.n0[0], td.n0[1], td.n0[2]);
	f3 n1 = mk3(td.n1[0], td.n1[1], td.n1[2]);
	f3 n2 = mk3(td.n2[0], td.n2[1], td.n2[2]);
	hi.normal = normalize3(add3(add3(n0, muls3(sub3(n1, n0), u)), muls3(sub3(n2, n0), v)));
	const uint32_t mi = td.materialIndex;
	const int4 tix = __ldg(reinterpret_cast<const int4*>(s.materials + mi));
	const float4 alb = __ldg(reinterpret_cast<const float4*>(s.materials + mi) + 1);
	const float4 rm = __ldg(reinterpret_cast<const float4*>(s.materials + mi) + 2);
	hi.albedo = mk3(alb.x, alb.y, alb.z);
	hi.alpha = alb.w;
	hi.roughness = rm.x;
	hi.metallic = rm.y;
	if ((tix.x & tix.y & tix.z) >= 0) {   // some texture index is set (indices are -1 or >= 0)
		// uv = uv0 + (uv1 - uv0) * u + (uv2 - uv0) * v, left to right
		float tu = __fadd_rn(__fadd_rn(td.uv0[0], __fmul_rn(__fsub_rn(td.uv1[0], td.uv0[0]), u)),
		                     __fmul_rn(__fsub_rn(td.uv2[0], td.uv0[0]), v));
		float tv = __fadd_rn(__fadd_rn(td.uv0[1], __fmul_rn(__fsub_rn(td.uv1[1], td.uv0[1]), u)),
		                     __fmul_rn(__fsub_rn(td.uv2[1], td.uv0[1]), v));
		if (tix.x >= 0) {
			uchar4 c = __ldg(reinterpret_cast<const uchar4*>(texel(s, tix.x, tu, tv)));
			hi.albedo = mk3(__ldg(s.srgb + c.x), __ldg(s.srgb + c.y), __ldg(s.srgb + c.z));
			hi.alpha = __fdiv_rn((float)c.w, 255.0f);
		}
		if (tix.y >= 0) hi.roughness = __fdiv_rn((float)__ldg(texel(s, tix.y, tu, tv)), 255.0f);
		if (tix.z >= 0) hi.metallic = __fdiv_rn((float)__ldg(texel(s, tix.z, tu, tv)), 255.0f);
	}
	return hi;
}

// One light of shadeHit: returns the contribution; when a shadow ray is to be cast, fills it and
// returns cast = true (random numbers are drawn only then, as in the reference).
__device__ __forceinline__ f3 shade_light(const phe_sphere_light& light, f3 mask, const HitInfo& hi, f3 toCamera,
                                          DevPcg& rng, bool& cast, f3& sdir, float& stmax)
{
	f3 lp = mk3(light.pos[0], light.pos[1], light.pos[2]);
	f3 toLight = sub3(lp, hi.pos);
	float toLightDist = length3(toLight);
	f3 l = divs3(toLight, toLightDist);
	float fo = falloff(toLightDist, light.range);
	f3 sh = shade(hi.normal, toCamera, hi.albedo, hi.roughness, hi.metallic, l, toLightDist,
	              mk3(light.strength[0], light.strength[1], light.strength[2]), light.range);
	f3 shading = mul3(muls3(mask, fo), sh);
	const float EPSILON = 0.0001f;
	bool contributes = shading.x > EPSILON || shading.y > EPSILON || shading.z > EPSILON;
	cast = light.staticShadows && contributes;
	if (cast) {
		f3 n = hi.normal;
		f3 circleU = fabsf(n.z) > 0.01f ? normalize3(mk3(0.0f, -n.z, n.y)) : normalize3(mk3(-n.y, n.x, 0.0f));
		f3 circleV = cross3(circleU, l);
		float r1 = rng.uniform();
		float r2 = rng.uniform();
		float centerDistance = __fmul_rn(light.radius, __fsub_rn(__fmul_rn(2.0f, r2), 1.0f));
		float s, c;
		sincos_2pi(r1, s, c);
		f3 offset = add3(muls3(muls3(circleU, c), centerDistance), muls3(muls3(circleV, s), centerDistance));
		f3 diff = sub3(add3(lp, offset), hi.pos);
		sdir = normalize3(diff);
		stmax = length3(diff);
	}
	return shading;
}

__device__ __forceinline__ f3 hemisphere_to_world(float cphi, float sphi, float cosTheta, float sinTheta, f3 normal)
{
	float hx = __fmul_rn(sinTheta, cphi), hy = __fmul_rn(sinTheta, sphi), hz = cosTheta;
	f3 up = fabsf(normal.z) < 0.999f ? mk3(0.0f, 0.0f, 1.0f) : mk3(1.0f, 0.0f, 0.0f);
	f3 u = normalize3(cross3(up, normal));
	f3 v = cross3(normal, u);
	return add3(add3(muls3(u, hx), muls3(v, hy)), muls3(normal, hz));
}

// Bounce ray of createSecondaryRaysKernel (MaterialKernel.cu:251-312) at full resolution from a
// primary hit: cosine-weighted when the roulette sample is below the roughness, GGX around the mirror
// direction otherwise; the glass branch for alpha <= 0.5. Returns the direction, tMin and throughput.
__device__ __forceinline__ f3 sample_bounce(const HitInfo& hi, f3 camPos, DevPcg& rng, float& tMin, f3& throughput)
{
	float r1 = rng.uniform();
	float r2 = rng.uniform();
	throughput = mk3(1.0f, 1.0f, 1.0f);
	tMin = 0.001f;
	f3 fromCamera = normalize3(sub3(hi.pos, camPos));
	f3 dir;
	if (hi.alpha > 0.5f) {
		float r3 = rng.uniform();
		throughput = mul3(throughput, hi.albedo);
		float s, c;
		sincos_2pi(r1, s, c);
		if (r3 < hi.roughness) {
			float sinTheta = __fsqrt_rn(r2);
			float cosTheta = __fsqrt_rn(__fsub_rn(1.0f, r2));
			dir = hemisphere_to_world(c, s, cosTheta, sinTheta, hi.normal);
		} else {
			f3 refl = sub3(fromCamera, muls3(hi.normal, __fmul_rn(2.0f, dot3(hi.normal, fromCamera))));
			float a = __fmul_rn(hi.roughness, hi.roughness);
			float cosTheta = __fsqrt_rn(__fdiv_rn(__fsub_rn(1.0f, r2),
			                                      __fadd_rn(1.0f, __fmul_rn(__fsub_rn(__fmul_rn(a, a), 1.0f), r2))));
			float sinTheta = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(cosTheta, cosTheta)));
			f3 vec = hemisphere_to_world(c, s, cosTheta, sinTheta, refl);
			float nDotV = dot3(vec, hi.normal);
			float off = -stdmin(0.0f, nDotV);
			dir = normalize3(add3(vec, muls3(hi.normal, off)));
		}
		throughput = muls3(throughput, 0.6f);
	} else {
		dir = normalize3(add3(muls3(fromCamera, 0.8f), muls3(mk3(-hi.normal.x, -hi.normal.y, -hi.normal.z), 0.2f)));
		tMin = 0.2f;
	}
	return dir;
}

} // namespace phe_gb300
