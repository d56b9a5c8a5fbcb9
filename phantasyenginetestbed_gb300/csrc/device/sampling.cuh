// GL-style sampling of float images in device memory, restated with explicit rounding so that the
// oracle reproduces it: GLSL mix() and GL_LINEAR filtering with clamp-to-edge addressing (the
// framebuffer textures of the reference's post-process passes, sfz/gl/Framebuffer.cpp:292-304).
#pragma once

#include <cstdint>

namespace phe_gb300 {

// GLSL mix(a, b, t) = a * (1 - t) + b * t
__device__ __forceinline__ float glsl_mix(float a, float b, float t)
{
	return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t));
}

// GL_LINEAR with clamp to edge at pixel-space position (px, py) measured from the texel grid origin
// (texel centres at integer + 0.5) of a W x H image of CH interleaved floats per texel.
template <int CH>
__device__ __forceinline__ void bilinear(const float* tex, uint32_t W, uint32_t H, float px, float py, float* out)
{
	float fx = __fsub_rn(px, 0.5f), fy = __fsub_rn(py, 0.5f);
	float x0f = floorf(fx), y0f = floorf(fy);
	float ax = __fsub_rn(fx, x0f), ay = __fsub_rn(fy, y0f);
	long x0 = (long)x0f, y0 = (long)y0f, x1 = x0 + 1, y1 = y0 + 1;
	long Wm = (long)W - 1, Hm = (long)H - 1;
	x0 = x0 < 0 ? 0 : (x0 > Wm ? Wm : x0);
	x1 = x1 < 0 ? 0 : (x1 > Wm ? Wm : x1);
	y0 = y0 < 0 ? 0 : (y0 > Hm ? Hm : y0);
	y1 = y1 < 0 ? 0 : (y1 > Hm ? Hm : y1);
	for (int c = 0; c < CH; c++) {
		float t00 = tex[((size_t)y0 * W + x0) * CH + c], t10 = tex[((size_t)y0 * W + x1) * CH + c];
		float t01 = tex[((size_t)y1 * W + x0) * CH + c], t11 = tex[((size_t)y1 * W + x1) * CH + c];
		out[c] = glsl_mix(glsl_mix(t00, t10, ax), glsl_mix(t01, t11, ax), ay);
	}
}

} // namespace phe_gb300
