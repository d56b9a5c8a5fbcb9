// Seeded synthetic scenes: heightfield + cubes. The reference renders Sponza, which is not in the
// reference tree; these scenes stand in for it with the shapes and sizes of the benchmark
// configurations. Every operation is IEEE double or float without contraction (the host library is
// built with -ffp-contract=off) and the sine is computed here, so x86-64 and aarch64 produce the
// same bytes.

#include <cmath>
#include <cstring>
#include <vector>

#include "common.hpp"
#include "pcg.hpp"

namespace phe_gb300 {
namespace {

// sin(x) in double: reduction by a multiple of pi/2 and Taylor series on [-pi/4, pi/4].
double det_sin(double x)
{
	const double HALF_PI = 1.5707963267948966;
	double k = std::nearbyint(x / HALF_PI);
	double r = x - k * HALF_PI;
	long q = (long)k;
	int quad = (int)(((q % 4) + 4) % 4);
	double r2 = r * r;
	// sin(r) = r - r^3/3! + ..., cos(r) = 1 - r^2/2! + ...; |r| <= pi/4, terms to r^17 / r^18.
	double s = 0.0, c = 0.0;
	{
		double term = r, acc = r;
		for (int n = 1; n <= 8; n++) {
			term = -term * r2 / (double)((2 * n) * (2 * n + 1));
			acc = acc + term;
		}
		s = acc;
	}
	{
		double term = 1.0, acc = 1.0;
		for (int n = 1; n <= 9; n++) {
			term = -term * r2 / (double)((2 * n - 1) * (2 * n));
			acc = acc + term;
		}
		c = acc;
	}
	switch (quad) {
	case 0: return s;
	case 1: return c;
	case 2: return -s;
	default: return -c;
	}
}
double det_cos(double x) { return det_sin(x + 1.5707963267948966); }

struct Octave { double f, ct, st, phi, w; };

struct Heightfield {
	Octave oct[4];
	double scale;
	double height(double xn, double yn) const
	{
		const double TWO_PI = 6.283185307179586;
		double h = 0.0;
		for (int k = 0; k < 4; k++) {
			const Octave& o = oct[k];
			h = h + o.w * det_sin(TWO_PI * o.f * (xn * o.ct + yn * o.st) + o.phi);
		}
		return scale * 0.1 * h / 1.875;
	}
};

struct V3 { float x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 crs(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 nrm(V3 a)
{
	float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
	return {a.x / l, a.y / l, a.z / l};
}

struct Writer {
	float* verts;
	phe_triangle_data* datas;
	phe_material* mats;
	Pcg32* matRng;
	uint64_t index = 0;
	void tri(V3 a, V3 b, V3 c)
	{
		if (verts) {
			float* p = verts + 9 * index;
			p[0] = a.x; p[1] = a.y; p[2] = a.z; p[3] = b.x; p[4] = b.y; p[5] = b.z; p[6] = c.x; p[7] = c.y; p[8] = c.z;
		}
		if (datas) {
			V3 n = nrm(crs(sub(b, a), sub(c, a)));
			phe_triangle_data& d = datas[index];
			std::memset(&d, 0, sizeof(d));
			d.n0[0] = d.n1[0] = d.n2[0] = n.x;
			d.n0[1] = d.n1[1] = d.n2[1] = n.y;
			d.n0[2] = d.n1[2] = d.n2[2] = n.z;
			d.materialIndex = (uint32_t)index;
		}
		if (mats) {
			phe_material& m = mats[index];
			std::memset(&m, 0, sizeof(m));
			for (int k = 0; k < 4; k++) m.texIndex[k] = -1;
			for (int k = 0; k < 3; k++) m.albedo[k] = 0.2f + 0.6f * matRng->uniform();
			m.albedo[3] = 1.0f;
			m.roughness = 1.0f;
			m.metallic = 0.0f;
		}
		index++;
	}
};

} // namespace
} // namespace phe_gb300

using namespace phe_gb300;

extern "C" uint64_t phe_scene_recipe_triangles(const phe_scene_recipe* r)
{
	if (!r) return 0;
	return 2ull * r->gridCells * r->gridCells + 12ull * r->numCubes;
}

extern "C" phe_status phe_scene_generate(const phe_scene_recipe* r, float* triVerts, phe_triangle_data* datas,
                                         phe_material* materials)
{
	if (!r || r->gridCells == 0) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_generate: empty recipe");
	if (phe_scene_recipe_triangles(r) > 0xFFFFFFF0ull)
		return fail(PHE_ERR_TOO_LARGE, "phe_scene_generate: more than 2^32 triangles");
	const uint32_t N = r->gridCells;
	const double TWO_PI = 6.283185307179586;
	Pcg32 rng(r->seed, 1);
	Pcg32 matRng(r->seed, 2);
	Heightfield hf;
	hf.scale = (double)N / 64.0;
	for (int k = 0; k < 4; k++) {
		double u = rng.uniform_d();
		double theta = TWO_PI * rng.uniform_d();
		double phi = TWO_PI * rng.uniform_d();
		hf.oct[k].f = (double)(1 << k) * (1.0 + u);
		hf.oct[k].ct = det_cos(theta);
		hf.oct[k].st = det_sin(theta);
		hf.oct[k].phi = phi;
		hf.oct[k].w = 1.0 / (double)(1 << k);
	}
	// Vertex heights on the (N+1)^2 grid; x = i/64, y = j/64 (exact in float).
	std::vector<float> h((size_t)(N + 1) * (N + 1));
	for (uint32_t j = 0; j <= N; j++)
		for (uint32_t i = 0; i <= N; i++)
			h[(size_t)j * (N + 1) + i] = (float)hf.height((double)i / N, (double)j / N);
	Writer w{triVerts, datas, materials, &matRng};
	for (uint32_t j = 0; j < N; j++)
		for (uint32_t i = 0; i < N; i++) {
			V3 v00 = {(float)i / 64.0f, (float)j / 64.0f, h[(size_t)j * (N + 1) + i]};
			V3 v10 = {(float)(i + 1) / 64.0f, (float)j / 64.0f, h[(size_t)j * (N + 1) + i + 1]};
			V3 v01 = {(float)i / 64.0f, (float)(j + 1) / 64.0f, h[(size_t)(j + 1) * (N + 1) + i]};
			V3 v11 = {(float)(i + 1) / 64.0f, (float)(j + 1) / 64.0f, h[(size_t)(j + 1) * (N + 1) + i + 1]};
			w.tri(v00, v10, v11);
			w.tri(v00, v11, v01);
		}
	// Cubes: edge U[0.01, 0.05] * scale, centre uniform over the heightfield, resting on it.
	for (uint32_t c = 0; c < r->numCubes; c++) {
		double e = (0.01 + 0.04 * rng.uniform_d()) * hf.scale;
		double cxn = rng.uniform_d(), cyn = rng.uniform_d();
		double cz = hf.height(cxn, cyn) + 0.5 * e;
		double cx = cxn * hf.scale, cy = cyn * hf.scale;
		// Rotation: identity or a uniform random unit quaternion (Shoemake 1992).
		double m[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
		if (r->rotatedCubes) {
			double u1 = rng.uniform_d(), u2 = rng.uniform_d(), u3 = rng.uniform_d();
			double a = std::sqrt(1.0 - u1), b = std::sqrt(u1);
			double qx = a * det_sin(TWO_PI * u2), qy = a * det_cos(TWO_PI * u2);
			double qz = b * det_sin(TWO_PI * u3), qw = b * det_cos(TWO_PI * u3);
			m[0][0] = 1 - 2 * (qy * qy + qz * qz); m[0][1] = 2 * (qx * qy - qz * qw); m[0][2] = 2 * (qx * qz + qy * qw);
			m[1][0] = 2 * (qx * qy + qz * qw); m[1][1] = 1 - 2 * (qx * qx + qz * qz); m[1][2] = 2 * (qy * qz - qx * qw);
			m[2][0] = 2 * (qx * qz - qy * qw); m[2][1] = 2 * (qy * qz + qx * qw); m[2][2] = 1 - 2 * (qx * qx + qy * qy);
		}
		V3 corner[8];
		for (int k = 0; k < 8; k++) {
			double lx = ((k & 1) ? 0.5 : -0.5) * e, ly = ((k & 2) ? 0.5 : -0.5) * e, lz = ((k & 4) ? 0.5 : -0.5) * e;
			corner[k].x = (float)(cx + m[0][0] * lx + m[0][1] * ly + m[0][2] * lz);
			corner[k].y = (float)(cy + m[1][0] * lx + m[1][1] * ly + m[1][2] * lz);
			corner[k].z = (float)(cz + m[2][0] * lx + m[2][1] * ly + m[2][2] * lz);
		}
		// Faces with outward winding (counter-clockwise seen from outside).
		static const int F[6][4] = {{0, 2, 3, 1}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 4, 6, 2}, {1, 3, 7, 5}};
		for (int f = 0; f < 6; f++) {
			w.tri(corner[F[f][0]], corner[F[f][1]], corner[F[f][2]]);
			w.tri(corner[F[f][0]], corner[F[f][2]], corner[F[f][3]]);
		}
	}
	return PHE_OK;
}
