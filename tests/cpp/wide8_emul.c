/* Test infrastructure: a scalar CPU emulation of the 8-wide compressed traversal (csrc/device/
 * traverse8.cuh) on the layout phe_bvh_wide8_build returns, with the same arithmetic: child boxes
 * decoded exactly from their grid bytes, slab distances with directed rounding (round down toward
 * the entry plane, up toward the exit plane) so that every quantized box test passes whenever the
 * reference's test of the exact box does, and each leaf's exact box re-tested with the reference
 * arithmetic before its triangles. Children are visited in the order of (slot XOR ray octant).
 * Directed rounding is computed exactly from round-to-nearest results and their error terms
 * (Knuth's two-sum, the fma product residual), so no floating-point environment is touched.
 * Used by tests/test_wide8.py to check the layout against the oracle on the CPU and to count the
 * nodes, leaves and triangles each ray visits. Built by that test with the host C compiler. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct { float o[3]; float tmin; float d[3]; float tmax; } ray_t;
typedef struct { uint32_t tri; float t, u, v; } hit_t;

static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static float sub_rd(float a, float b)
{
	float c = -b, s = a + c, bb = s - a;
	float e = (a - (s - bb)) + (c - bb);
	if (isinf(s)) return s > 0 ? FLT_MAX : s;
	return e < 0.0f ? nextafterf(s, -INFINITY) : s;
}
static float sub_ru(float a, float b)
{
	float c = -b, s = a + c, bb = s - a;
	float e = (a - (s - bb)) + (c - bb);
	if (isinf(s)) return s < 0 ? -FLT_MAX : s;
	return e > 0.0f ? nextafterf(s, INFINITY) : s;
}
static float mul_rd(float a, float b)
{
	float r = a * b, e = fmaf(a, b, -r);
	return e < 0.0f ? nextafterf(r, -INFINITY) : r;
}
static float mul_ru(float a, float b)
{
	float r = a * b, e = fmaf(a, b, -r);
	return e > 0.0f ? nextafterf(r, INFINITY) : r;
}

/* Intersection.hpp:24-67 on a TriangleVertices slot (v0, v1, v2 as 4 floats each). */
static int tri_test(const float* tv, const float* o, const float* d, float* t, float* u, float* v)
{
	const float EPS = 0.00001f;
	float e1[3] = {tv[4] - tv[0], tv[5] - tv[1], tv[6] - tv[2]};
	float e2[3] = {tv[8] - tv[0], tv[9] - tv[1], tv[10] - tv[2]};
	float q[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
	float a = e1[0] * q[0] + e1[1] * q[1] + e1[2] * q[2];
	if (-EPS < a && a < EPS) return 0;
	float f = 1.0f / a;
	float s[3] = {o[0] - tv[0], o[1] - tv[1], o[2] - tv[2]};
	float uu = f * (s[0] * q[0] + s[1] * q[1] + s[2] * q[2]);
	if (uu < 0.0f) return 0;
	float r[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2], s[0] * e1[1] - s[1] * e1[0]};
	float vv = f * (d[0] * r[0] + d[1] * r[1] + d[2] * r[2]);
	if (vv < 0.0f || uu + vv > 1.0f) return 0;
	*t = f * (e2[0] * r[0] + e2[1] * r[1] + e2[2] * r[2]);
	*u = uu;
	*v = vv;
	return 1;
}

static uint32_t perm8(uint32_t m, uint32_t oct)
{
	if (oct & 1) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
	if (oct & 2) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
	if (oct & 4) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
	return m;
}

static uint32_t rank(uint32_t mask, uint32_t s) { return (uint32_t)__builtin_popcount(mask & ((1u << s) - 1u)); }

typedef struct { uint32_t base, mask, keys, leaf; } group_t;

#define STACK 160

/* mode 0: closest hit (accept tMin <= t < current), 1: any hit. stats (optional): 3 per ray: nodes
 * intersected, leaf records tested, triangle tests. Returns the number of rays that overflowed. */
int wide8_cast(const uint32_t* nodes, const float* leaves, const float* tris, const ray_t* rays, uint32_t n, int mode,
               hit_t* hits, uint8_t* inLight, uint32_t* stats)
{
	int overflows = 0;
	for (uint32_t i = 0; i < n; i++) {
		const ray_t* r = &rays[i];
		float inv[3], a[3], so[3], sg[3];
		uint32_t oct = 0;
		for (int k = 0; k < 3; k++) {
			inv[k] = 1.0f / r->d[k];
			a[k] = fabsf(inv[k]);
			sg[k] = r->d[k] < 0.0f ? -1.0f : 1.0f;
			so[k] = sg[k] * r->o[k];
			if (r->d[k] < 0.0f) oct |= 1u << k;
		}
		hit_t h = {~0u, fminf(r->tmax, FLT_MAX), 0.0f, 0.0f};
		uint32_t cn = 0, cl = 0, ct = 0;
		group_t stack[STACK];
		int sp = 0, done = 0;
		group_t g = {0, 0, 0, 0};
		int32_t node = 0;
		while (!done) {
			if (node >= 0) {
				/* intersect one node */
				const uint32_t* w = nodes + 20 * (size_t)node;
				cn++;
				uint32_t meta = w[3], imask = meta >> 24, valid = w[6];
				float sp3[3], ss3[3];
				const uint8_t* nb[3];
				const uint8_t* fb[3];
				for (int k = 0; k < 3; k++) {
					int e = (int)((meta >> (8 * k)) & 0xFFu) - 128;
					float s = ldexpf(1.0f, e);
					sp3[k] = sg[k] * u2f(w[k]);
					ss3[k] = sg[k] * s;
					const uint8_t* lo = (const uint8_t*)(w + 8 + 4 * k);
					nb[k] = sg[k] > 0 ? lo : lo + 8;
					fb[k] = sg[k] > 0 ? lo + 8 : lo;
				}
				uint32_t hitS = 0;
				for (int c = 0; c < 8; c++) {
					float tin = -INFINITY, tout = INFINITY;
					for (int k = 0; k < 3; k++) {
						float bn = fmaf(8388608.0f + (float)nb[k][c], ss3[k], sp3[k]);
						float bf = fmaf(8388608.0f + (float)fb[k][c], ss3[k], sp3[k]);
						float tn = mul_rd(sub_rd(bn, so[k]), a[k]);
						float tf = mul_ru(sub_ru(bf, so[k]), a[k]);
						tin = fmaxf(tin, tn);
						tout = fminf(tout, tf);
					}
					if (tout >= tin && tout > r->tmin && tin < h.t) hitS |= 1u << c;
				}
				hitS &= valid;
				uint32_t keys = perm8(hitS, oct), ikeys = perm8(imask, oct);
				uint32_t li = keys & ~ikeys, ni = keys & ikeys;
				node = -1;
				if (ni) {
					if (sp >= STACK) { overflows++; done = 1; break; }
					stack[sp++] = (group_t){w[4], imask, ni, 0};
				}
				if (li) g = (group_t){w[5], valid & ~imask, li, 1};
				else g.keys = 0;
			}
			/* leaves of the current leaf group, in key order */
			while (g.leaf && g.keys && !done) {
				uint32_t k = (uint32_t)__builtin_ctz(g.keys);
				g.keys &= g.keys - 1u;
				uint32_t s = k ^ oct;
				const float* rec = leaves + 8 * (size_t)(g.base + rank(g.mask, s));
				uint32_t first, count;
				memcpy(&first, &rec[3], 4);
				memcpy(&count, &rec[7], 4);
				cl++;
				/* exact box (Intersection.hpp:77-90) and the visit rule of BVHTraversal.hpp:152-156 */
				float t1[3], t2[3];
				for (int q = 0; q < 3; q++) {
					t1[q] = (rec[q] - r->o[q]) * inv[q];
					t2[q] = (rec[4 + q] - r->o[q]) * inv[q];
				}
				float tmn = fmaxf(fmaxf(fminf(t1[0], t2[0]), fminf(t1[1], t2[1])), fminf(t1[2], t2[2]));
				float tmx = fminf(fminf(fmaxf(t1[0], t2[0]), fmaxf(t1[1], t2[1])), fmaxf(t1[2], t2[2]));
				if (!(tmx >= tmn && tmx > r->tmin && tmn < h.t)) continue;
				for (uint32_t j = 0; j < count; j++) {
					float t, u, v;
					ct++;
					if (tri_test(tris + 12 * (size_t)(first + j), r->o, r->d, &t, &u, &v) && r->tmin <= t && t < h.t) {
						h.tri = first + j; h.t = t; h.u = u; h.v = v;
						if (mode == 1) { done = 1; break; }
					}
				}
			}
			if (done) break;
			/* next node: lowest key of the top node group */
			while (node < 0) {
				if (sp == 0) { done = 1; break; }
				group_t* top = &stack[sp - 1];
				uint32_t k = (uint32_t)__builtin_ctz(top->keys);
				top->keys &= top->keys - 1u;
				uint32_t s = k ^ oct;
				node = (int32_t)(top->base + rank(top->mask, s));
				if (!top->keys) sp--;
			}
		}
		if (h.tri == ~0u) { h.t = r->tmax; h.u = 0.0f; h.v = 0.0f; }
		if (hits) hits[i] = h;
		if (inLight) inLight[i] = h.tri == ~0u;
		if (stats) { stats[3 * i] = cn; stats[3 * i + 1] = cl; stats[3 * i + 2] = ct; }
	}
	return overflows;
}
