// Drives the reference-signature launch functions (include/phe_reference_api.hpp) the way the
// reference's renderer does: scene arrays uploaded into float4 linear texture objects exactly as
// CudaTextureBuffer creates them (cuda_ray_tracer/CudaTextureBuffer.hpp:45-69), rays in a device
// buffer, synchronous launches. Reads <dir>/nodes.bin, verts.bin, rays.bin and a camera def, writes
// closest.bin, plain.bin, shadow.bin and primary.bin for the Python test to compare with the oracle.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "phe_reference_api.hpp"

static std::vector<char> readFile(const std::string& p)
{
	FILE* f = std::fopen(p.c_str(), "rb");
	if (!f) { std::fprintf(stderr, "cannot open %s\n", p.c_str()); std::exit(2); }
	std::fseek(f, 0, SEEK_END);
	long n = std::ftell(f);
	std::fseek(f, 0, SEEK_SET);
	std::vector<char> b((size_t)n);
	if (n && std::fread(b.data(), 1, (size_t)n, f) != (size_t)n) std::exit(2);
	std::fclose(f);
	return b;
}

static void writeFile(const std::string& p, const void* d, size_t n)
{
	FILE* f = std::fopen(p.c_str(), "wb");
	if (!f || std::fwrite(d, 1, n, f) != n) std::exit(3);
	std::fclose(f);
}

static cudaTextureObject_t linearFloat4Texture(const std::vector<char>& host, void** devOut)
{
	void* dev = nullptr;
	if (cudaMalloc(&dev, host.size()) != cudaSuccess) std::exit(4);
	cudaMemcpy(dev, host.data(), host.size(), cudaMemcpyHostToDevice);
	cudaResourceDesc resDesc;
	std::memset(&resDesc, 0, sizeof(resDesc));
	resDesc.resType = cudaResourceTypeLinear;
	resDesc.res.linear.devPtr = dev;
	resDesc.res.linear.desc.f = cudaChannelFormatKindFloat;
	resDesc.res.linear.desc.x = 32;
	resDesc.res.linear.desc.y = 32;
	resDesc.res.linear.desc.z = 32;
	resDesc.res.linear.desc.w = 32;
	resDesc.res.linear.sizeInBytes = host.size();
	cudaTextureDesc texDesc;
	std::memset(&texDesc, 0, sizeof(texDesc));
	texDesc.readMode = cudaReadModeElementType;
	cudaTextureObject_t tex = 0;
	if (cudaCreateTextureObject(&tex, &resDesc, &texDesc, nullptr) != cudaSuccess) std::exit(5);
	*devOut = dev;
	return tex;
}

int main(int argc, char** argv)
{
	if (argc < 2) return 1;
	std::string dir = argv[1];
	std::vector<char> nodes = readFile(dir + "/nodes.bin"), verts = readFile(dir + "/verts.bin");
	std::vector<char> rays = readFile(dir + "/rays.bin"), camRes = readFile(dir + "/camera.bin");
	void *dNodes, *dVerts;
	phe::RayCastKernelInput in;
	in.bvhNodes = linearFloat4Texture(nodes, &dNodes);
	in.triangleVerts = linearFloat4Texture(verts, &dVerts);
	in.numRays = (uint32_t)(rays.size() / sizeof(phe::RayIn));
	phe::RayIn* dRays = nullptr;
	phe::RayHit* dHits = nullptr;
	bool* dLight = nullptr;
	cudaMalloc(&dRays, rays.size());
	cudaMalloc(&dHits, in.numRays * sizeof(phe::RayHit));
	cudaMalloc(&dLight, in.numRays);
	cudaMemcpy(dRays, rays.data(), rays.size(), cudaMemcpyHostToDevice);
	in.rays = dRays;
	cudaDeviceProp prop;
	cudaGetDeviceProperties(&prop, 0);

	std::vector<char> out(in.numRays * sizeof(phe::RayHit));
	phe::launchRayCastKernel(in, dHits, prop);
	cudaMemcpy(out.data(), dHits, out.size(), cudaMemcpyDeviceToHost);
	writeFile(dir + "/closest.bin", out.data(), out.size());
	cudaMemset(dHits, 0xAB, out.size());
	phe::launchRayCastNoPersistenceKernel(in, dHits, prop);
	cudaMemcpy(out.data(), dHits, out.size(), cudaMemcpyDeviceToHost);
	writeFile(dir + "/plain.bin", out.data(), out.size());
	phe::launchShadowRayCastKernel(in, dLight, prop);
	std::vector<char> lit(in.numRays);
	cudaMemcpy(lit.data(), dLight, lit.size(), cudaMemcpyDeviceToHost);
	writeFile(dir + "/shadow.bin", lit.data(), lit.size());

	// camera.bin: 12 floats of CameraDef + 2 int32 resolution
	phe::CameraDef cam;
	std::memcpy(&cam, camRes.data(), sizeof(cam));
	phe::ApiVec2i res;
	std::memcpy(&res, camRes.data() + sizeof(cam), sizeof(res));
	phe::RayIn* dPrimary = nullptr;
	size_t np = (size_t)res.x * res.y;
	cudaMalloc(&dPrimary, np * sizeof(phe::RayIn));
	phe::launchGenPrimaryRaysKernel(dPrimary, cam, res);
	std::vector<char> prim(np * sizeof(phe::RayIn));
	cudaMemcpy(prim.data(), dPrimary, prim.size(), cudaMemcpyDeviceToHost);
	writeFile(dir + "/primary.bin", prim.data(), prim.size());

	// A second call on the same texture objects reuses the cached scene.
	phe::launchRayCastKernel(in, dHits, prop);
	std::vector<char> again(out.size());
	cudaMemcpy(again.data(), dHits, again.size(), cudaMemcpyDeviceToHost);
	int same = std::memcmp(again.data(), readFile(dir + "/closest.bin").data(), again.size()) == 0;
	phe::invalidateSceneCache();
	cudaDestroyTextureObject(in.bvhNodes);
	cudaDestroyTextureObject(in.triangleVerts);
	cudaFree(dNodes); cudaFree(dVerts); cudaFree(dRays); cudaFree(dHits); cudaFree(dLight); cudaFree(dPrimary);
	std::printf("reference_api_test: %u rays, repeat identical: %d\n", in.numRays, same);
	return same ? 0 : 6;
}
