// Display post-process for headless image dumps: the Uncharted 2 filmic tonemap followed by gamma
// correction (resources/shaders/gamma_correction.frag:20-74, the combination its main() selects), from
// a linear float RGBA image to display-referred float RGBA and/or 8-bit RGBA. The GL pass drew into a
// window; here the result is a device buffer the caller copies out (or writes to a file).

#include "runtime.cuh"
#include "sampling.cuh"

namespace phe_gb300 {

// gamma_correction.frag:35-43 constants; products of constants are folded in float as GLSL does.
__device__ __forceinline__ float u2(float x)
{
	const float A = 0.25f, B = 0.25f, C = 0.105f, D = 0.20f, E = 0.025f, F = 0.25f;
	float num = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(A, x), __fmul_rn(C, B))), __fmul_rn(D, E));
	float den = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(A, x), B)), __fmul_rn(D, F));
	return __fsub_rn(__fdiv_rn(num, den), __fdiv_rn(E, F));
}

__device__ __forceinline__ unsigned char to_byte(float v)
{
	return (unsigned char)__float2int_rn(__fmul_rn(fminf(fmaxf(v, 0.0f), 1.0f), 255.0f));
}

__global__ void postprocess_kernel(uint32_t n, const float4* __restrict__ linear, float invGamma,
                                   float4* __restrict__ display, uchar4* __restrict__ rgba8)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	float4 c = linear[i];
	const float W = 11.2f, BLACK_CRUSH = 0.0015f, exposureBias = 2.0f;
	float white = u2(W);
	float v[3] = {c.x, c.y, c.z};
	for (int k = 0; k < 3; k++) {
		float x = __fmul_rn(exposureBias, fmaxf(0.0f, __fsub_rn(v[k], BLACK_CRUSH)));
		v[k] = powf(__fdiv_rn(u2(x), white), invGamma);
	}
	if (display) display[i] = make_float4(v[0], v[1], v[2], c.w);
	if (rgba8) {
		unsigned char q[4];
		float a[4] = {v[0], v[1], v[2], c.w};
		for (int k = 0; k < 4; k++) q[k] = to_byte(a[k]);
		rgba8[i] = make_uchar4(q[0], q[1], q[2], q[3]);
	}
}

// scaling.frag:19-35 for destination pixel (x, y): uv at the pixel centre, coord = uv * viewport / src,
// four GL_LINEAR taps at +-1/4 destination pixel, averaged; alpha 1.
__global__ void scale_kernel(uint32_t srcW, uint32_t srcH, const float4* __restrict__ src, float vpW, float vpH,
                             uint32_t dstW, uint32_t dstH, float4* __restrict__ dst, uchar4* __restrict__ rgba8)
{
	uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= dstW || y >= dstH) return;
	const float dw = (float)dstW, dh = (float)dstH, sw = (float)srcW, sh = (float)srcH;
	float u = __fdiv_rn(__fadd_rn((float)x, 0.5f), dw), v = __fdiv_rn(__fadd_rn((float)y, 0.5f), dh);
	float ox = __fmul_rn(__fdiv_rn(1.0f, dw), 0.25f), oy = __fmul_rn(__fdiv_rn(1.0f, dh), 0.25f);
	float cx = __fdiv_rn(__fmul_rn(u, vpW), sw), cy = __fdiv_rn(__fmul_rn(v, vpH), sh);
	const float sx[4] = {-ox, ox, -ox, ox}, sy[4] = {-oy, -oy, oy, oy};
	float acc[3] = {0.0f, 0.0f, 0.0f};
	for (int k = 0; k < 4; k++) {
		float t[4];
		bilinear<4>(reinterpret_cast<const float*>(src), srcW, srcH, __fmul_rn(__fadd_rn(cx, sx[k]), sw),
		            __fmul_rn(__fadd_rn(cy, sy[k]), sh), t);
		for (int c = 0; c < 3; c++) acc[c] = k == 0 ? t[c] : __fadd_rn(acc[c], t[c]);
	}
	float4 o = make_float4(__fdiv_rn(acc[0], 4.0f), __fdiv_rn(acc[1], 4.0f), __fdiv_rn(acc[2], 4.0f), 1.0f);
	size_t p = (size_t)y * dstW + x;
	if (dst) dst[p] = o;
	if (rgba8) rgba8[p] = make_uchar4(to_byte(o.x), to_byte(o.y), to_byte(o.z), 255);
}

} // namespace phe_gb300

using namespace phe_gb300;

extern "C" phe_status phe_scale(uint32_t srcW, uint32_t srcH, const float* src, uint32_t viewportW, uint32_t viewportH,
                                uint32_t dstW, uint32_t dstH, float* dst, uint8_t* dstRgba8, void* stream)
{
	if (!src || (!dst && !dstRgba8)) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scale: null buffer");
	if (!srcW || !srcH || !viewportW || !viewportH || viewportW > srcW || viewportH > srcH)
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scale: viewport must be a non-empty part of the source");
	if (srcW > 65536 || srcH > 65536 || dstW > 65536 || dstH > 65536)
		return fail(PHE_ERR_TOO_LARGE, "phe_scale: images are limited to 65536 x 65536");
	if (!dstW || !dstH) return PHE_OK;
	dim3 block(16, 8);
	dim3 grid((dstW + 15) / 16, (dstH + 7) / 8);
	scale_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(srcW, srcH, (const float4*)src, (float)viewportW,
	                                                      (float)viewportH, dstW, dstH, (float4*)dst, (uchar4*)dstRgba8);
	PHE_CUDA_TRY(cudaGetLastError(), "scale_kernel launch");
	return PHE_OK;
}

extern "C" phe_status phe_postprocess(uint32_t resX, uint32_t resY, const float* linear, float gamma, float* display,
                                      uint8_t* rgba8, void* stream)
{
	if (!linear || (!display && !rgba8)) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_postprocess: null buffer");
	if (!(gamma > 0.0f)) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_postprocess: gamma must be positive");
	uint64_t n = (uint64_t)resX * resY;
	if (n == 0) return PHE_OK;
	if (n > 0xFFFFFFFFull) return fail(PHE_ERR_TOO_LARGE, "phe_postprocess: too many pixels");
	uint32_t grid = (uint32_t)((n + 255) / 256);
	postprocess_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((uint32_t)n, (const float4*)linear, 1.0f / gamma,
	                                                          (float4*)display, (uchar4*)rgba8);
	PHE_CUDA_TRY(cudaGetLastError(), "postprocess_kernel launch");
	return PHE_OK;
}
