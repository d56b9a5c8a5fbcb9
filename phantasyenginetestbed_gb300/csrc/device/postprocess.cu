// Display post-process for headless image dumps: the Uncharted 2 filmic tonemap followed by gamma
// correction (resources/shaders/gamma_correction.frag:20-74, the combination its main() selects), from
// a linear float RGBA image to display-referred float RGBA and/or 8-bit RGBA. The GL pass drew into a
// window; here the result is a device buffer the caller copies out (or writes to a file).

#include "runtime.cuh"

namespace phe_gb300 {

// gamma_correction.frag:35-43 constants; products of constants are folded in float as GLSL does.
__device__ __forceinline__ float u2(float x)
{
	const float A = 0.25f, B = 0.25f, C = 0.105f, D = 0.20f, E = 0.025f, F = 0.25f;
	float num = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(A, x), __fmul_rn(C, B))), __fmul_rn(D, E));
	float den = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(A, x), B)), __fmul_rn(D, F));
	return __fsub_rn(__fdiv_rn(num, den), __fdiv_rn(E, F));
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
		for (int k = 0; k < 4; k++) q[k] = (unsigned char)__float2int_rn(__fmul_rn(fminf(fmaxf(a[k], 0.0f), 1.0f), 255.0f));
		rgba8[i] = make_uchar4(q[0], q[1], q[2], q[3]);
	}
}

} // namespace phe_gb300

using namespace phe_gb300;

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
