/* Test infrastructure only (the oracle): a plain-C restatement of the reference's ray-cast,
 * shading and TAA arithmetic. See oracle.h for the contract. Built by oracle/Makefile with
 * -ffp-contract=off and without -ffast-math; every expression keeps the reference's operation
 * order (sfz vector math is left-to-right: dot = x*x' + y*y' + z*z', Vector.inl:345-350;
 * cross Vector.inl:362-366; normalize = v / sqrt(dot(v, v)), Vector.inl:312-317). */
#define _GNU_SOURCE
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------------------------------
 * Vector helpers in sfz order
 * ------------------------------------------------------------------------------------------- */

typedef struct { float x, y, z; } v3;

static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 muls(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 divs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline v3 divv(v3 a, v3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b)
{
	return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float length3(v3 a) { return sqrtf(dot(a, a)); }
static inline v3 normalize3(v3 a) { return divs(a, length3(a)); }
/* std::min / std::max (the reference's sfz::min/max/minElement/maxElement use them). */
static inline float stdmin(float a, float b) { return (b < a) ? b : a; }
static inline float stdmax(float a, float b) { return (a < b) ? b : a; }

/* ---------------------------------------------------------------------------------------------
 * Intersection.hpp:24-67 and :77-90
 * ------------------------------------------------------------------------------------------- */

int oracle_intersect_tri(const or_tri* tri, const float o[3], const float d[3], float* t, float* u, float* v)
{
	const float EPS = 0.00001f;
	v3 p0 = ld3(tri->v0), p1 = ld3(tri->v1), p2 = ld3(tri->v2);
	v3 dir = ld3(d), origin = ld3(o);
	v3 e1 = sub(p1, p0);
	v3 e2 = sub(p2, p0);
	v3 q = cross(dir, e2);
	float a = dot(e1, q);
	if (-EPS < a && a < EPS) return 0;
	float f = 1.0f / a;
	v3 s = sub(origin, p0);
	float uu = f * dot(s, q);
	if (uu < 0.0f) return 0;
	v3 r = cross(s, e1);
	float vv = f * dot(dir, r);
	if (vv < 0.0f || (uu + vv) > 1.0f) return 0;
	*t = f * dot(e2, r);
	*u = uu;
	*v = vv;
	return 1;
}

typedef struct { int hit; float tIn, tOut; } aabb_hit;

static inline aabb_hit intersect_aabb(v3 origin, v3 invDir, v3 mn, v3 mx)
{
	v3 t1 = mulv(sub(mn, origin), invDir);
	v3 t2 = mulv(sub(mx, origin), invDir);
	float tmin = stdmax(stdmax(stdmin(t1.x, t2.x), stdmin(t1.y, t2.y)), stdmin(t1.z, t2.z));
	float tmax = stdmin(stdmin(stdmax(t1.x, t2.x), stdmax(t1.y, t2.y)), stdmax(t1.z, t2.z));
	aabb_hit h;
	h.hit = tmax >= tmin;
	h.tIn = tmin;
	h.tOut = tmax;
	return h;
}

/* ---------------------------------------------------------------------------------------------
 * castRay / castDebugRay (BVHTraversal.hpp:37-235)
 * ------------------------------------------------------------------------------------------- */

#define OR_STACK 144

int oracle_cast_ray(const or_node* nodes, const or_tri* tris, const or_ray* ray, int mode, or_hit* out,
                    uint32_t* nodesVisited, uint32_t* triTests)
{
	v3 origin = ld3(ray->o), dir = ld3(ray->d);
	v3 invDir = divv(mk(1.0f, 1.0f, 1.0f), dir); /* Ray::setDir, Ray.hpp:34-37 */
	const float tMin = ray->tmin, tMax = ray->tmax;
	uint32_t stack[OR_STACK];
	uint32_t stackSize = 1;
	stack[0] = 0;
	uint32_t bestTri = ~0u;
	float bestT, bestU, bestV;
	if (mode == OR_MODE_REFERENCE_CPU) {
		bestT = FLT_MAX; bestU = FLT_MAX; bestV = FLT_MAX;
	} else {
		bestT = stdmin(tMax, FLT_MAX); bestU = 0.0f; bestV = 0.0f;
	}
	uint32_t nv = 0, nt = 0;
	int overflow = 0;

	while (stackSize > 0) {
		stackSize--;
		const or_node* node = &nodes[stack[stackSize]];
		nv++;
		aabb_hit lc = intersect_aabb(origin, invDir, mk(node->f[0], node->f[1], node->f[2]),
		                             mk(node->f[3], node->f[4], node->f[5]));
		aabb_hit rc = intersect_aabb(origin, invDir, mk(node->f[6], node->f[7], node->f[8]),
		                             mk(node->f[9], node->f[10], node->f[11]));
		float tCurrMax = stdmin(tMax, bestT);
		int visit[2];
		visit[0] = lc.hit && lc.tOut > tMin && lc.tIn < tCurrMax;
		visit[1] = rc.hit && rc.tOut > tMin && rc.tIn < tCurrMax;
		for (int c = 0; c < 2; c++) {
			if (!visit[c]) continue;
			int32_t raw = node->i[c];
			uint32_t idx = (uint32_t)(raw < 0 ? ~raw : raw);
			uint32_t numTris = (uint32_t)node->i[2 + c];
			if (numTris == 0) {
				if (stackSize >= OR_STACK) { overflow = 1; continue; }
				stack[stackSize++] = idx;
			} else {
				for (uint32_t i = 0; i < numTris; i++) {
					float t, u, v;
					nt++;
					if (!oracle_intersect_tri(&tris[idx + i], ray->o, ray->d, &t, &u, &v)) continue;
					int accept = (mode == OR_MODE_REFERENCE_CPU)
					                 ? (t < bestT && tMin <= t && t <= tMax)
					                 : (tMin <= t && t < bestT);
					if (accept) {
						bestTri = idx + i; bestT = t; bestU = u; bestV = v;
					}
				}
			}
		}
	}
	out->tri = bestTri;
	out->t = bestT;
	out->u = bestU;
	out->v = bestV;
	if (mode == OR_MODE_REFERENCE_GPU && bestTri == ~0u) {
		out->t = tMax; out->u = 0.0f; out->v = 0.0f;
	}
	if (nodesVisited) *nodesVisited = nv;
	if (triTests) *triTests = nt;
	return overflow ? -1 : 0;
}

/* ---------------------------------------------------------------------------------------------
 * Threaded batches
 * ------------------------------------------------------------------------------------------- */

typedef struct {
	const or_node* nodes; const or_tri* tris; const or_ray* rays; uint32_t n; int mode;
	or_hit* hits; uint32_t* debug; uint8_t* inLight;
	atomic_uint next; atomic_int overflows;
} batch_job;

#define OR_CHUNK 64u

static void* batch_worker(void* arg)
{
	batch_job* j = (batch_job*)arg;
	for (;;) {
		uint32_t b = atomic_fetch_add(&j->next, OR_CHUNK);
		if (b >= j->n) break;
		uint32_t e = b + OR_CHUNK < j->n ? b + OR_CHUNK : j->n;
		for (uint32_t i = b; i < e; i++) {
			or_hit h;
			uint32_t nv, nt;
			int rc = oracle_cast_ray(j->nodes, j->tris, &j->rays[i], j->mode, &h, &nv, &nt);
			if (rc) atomic_fetch_add(&j->overflows, 1);
			if (j->hits) j->hits[i] = h;
			if (j->inLight) j->inLight[i] = (h.tri == ~0u) ? 1 : 0;
			if (j->debug) { j->debug[2 * (size_t)i] = nv; j->debug[2 * (size_t)i + 1] = nt; }
		}
	}
	return NULL;
}

static int run_batch(batch_job* j, int threads)
{
	atomic_init(&j->next, 0u);
	atomic_init(&j->overflows, 0);
	if (threads < 1) threads = 1;
	if (threads == 1 || j->n < 2 * OR_CHUNK) {
		batch_worker(j);
	} else {
		pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
		int started = 0;
		for (int t = 0; t < threads; t++)
			if (pthread_create(&th[t], NULL, batch_worker, j) == 0) started++;
			else break;
		if (started == 0) batch_worker(j);
		for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
		free(th);
	}
	return atomic_load(&j->overflows);
}

int oracle_cast_rays(const or_node* nodes, const or_tri* tris, const or_ray* rays, uint32_t n, int mode,
                     or_hit* hits, uint32_t* debug, int threads)
{
	batch_job j;
	memset(&j, 0, sizeof(j));
	j.nodes = nodes; j.tris = tris; j.rays = rays; j.n = n; j.mode = mode; j.hits = hits; j.debug = debug;
	return run_batch(&j, threads);
}

int oracle_any_rays(const or_node* nodes, const or_tri* tris, const or_ray* rays, uint32_t n,
                    uint8_t* inLight, int threads)
{
	batch_job j;
	memset(&j, 0, sizeof(j));
	j.nodes = nodes; j.tris = tris; j.rays = rays; j.n = n; j.mode = OR_MODE_REFERENCE_GPU; j.inLight = inLight;
	return run_batch(&j, threads);
}

void oracle_brute_closest(const or_tri* tris, uint32_t numTris, const or_ray* rays, uint32_t n, int mode,
                          or_hit* hits)
{
	for (uint32_t i = 0; i < n; i++) {
		const or_ray* r = &rays[i];
		or_hit h;
		h.tri = ~0u;
		if (mode == OR_MODE_REFERENCE_CPU) { h.t = FLT_MAX; h.u = FLT_MAX; h.v = FLT_MAX; }
		else { h.t = stdmin(r->tmax, FLT_MAX); h.u = 0.0f; h.v = 0.0f; }
		for (uint32_t s = 0; s < numTris; s++) {
			float t, u, v;
			if (!oracle_intersect_tri(&tris[s], r->o, r->d, &t, &u, &v)) continue;
			int accept = (mode == OR_MODE_REFERENCE_CPU) ? (t < h.t && r->tmin <= t && t <= r->tmax)
			                                             : (r->tmin <= t && t < h.t);
			if (accept) { h.tri = s; h.t = t; h.u = u; h.v = v; }
		}
		if (mode == OR_MODE_REFERENCE_GPU && h.tri == ~0u) h.t = r->tmax;
		hits[i] = h;
	}
}

/* ---------------------------------------------------------------------------------------------
 * Camera and primary rays
 * ------------------------------------------------------------------------------------------- */

void oracle_camera_def(const float pos[3], const float dir[3], const float up[3], float vfovRad,
                       float resX, float resY, or_camera* out)
{
	v3 camDir = normalize3(ld3(dir));
	v3 camUp = normalize3(ld3(up));
	v3 camRight = normalize3(cross(camDir, camUp));
	float aspect = resX / resY;
	float yMaxOffset = tanf(vfovRad * 0.5f);
	float xMaxOffset = aspect * yMaxOffset;
	v3 dX = muls(camRight, xMaxOffset), dY = muls(camUp, yMaxOffset);
	memcpy(out->origin, pos, 12);
	out->dir[0] = camDir.x; out->dir[1] = camDir.y; out->dir[2] = camDir.z;
	out->dX[0] = dX.x; out->dX[1] = dX.y; out->dX[2] = dX.z;
	out->dY[0] = dY.x; out->dY[1] = dY.y; out->dY[2] = dY.z;
}

uint32_t oracle_ray_index(uint32_t x, uint32_t y, uint32_t resX, int order)
{
	if (order == 0) return y * resX + x;
	uint32_t pixBlockIdx = (y / 8u) * (resX / 8u) + (x / 8u);
	return pixBlockIdx * 64u + (y % 8u) * 8u + (x % 8u);
}

static v3 primary_dir(const or_camera* cam, float lx, float ly, float resX, float resY)
{
	float nx = lx / resX, ny = ly / resY;
	float cx = nx * 2.0f - 1.0f, cy = ny * 2.0f - 1.0f;
	v3 nonNorm = add(add(ld3(cam->dir), muls(ld3(cam->dX), cx)), muls(ld3(cam->dY), cy));
	return normalize3(nonNorm);
}

void oracle_gen_primary(const or_camera* cam, uint32_t resX, uint32_t resY, float jx, float jy, int order,
                        or_ray* rays)
{
	for (uint32_t y = 0; y < resY; y++)
		for (uint32_t x = 0; x < resX; x++) {
			v3 d = primary_dir(cam, (float)x + jx, (float)y + jy, (float)resX, (float)resY);
			or_ray* r = &rays[oracle_ray_index(x, y, resX, order)];
			r->o[0] = cam->origin[0]; r->o[1] = cam->origin[1]; r->o[2] = cam->origin[2];
			r->tmin = 0.0001f;
			r->d[0] = d.x; r->d[1] = d.y; r->d[2] = d.z;
			r->tmax = FLT_MAX;
		}
}

/* ---------------------------------------------------------------------------------------------
 * PCG32 and the sine/cosine used for sampling
 * ------------------------------------------------------------------------------------------- */

static const uint64_t PCG_MULT = 6364136223846793005ull;

uint32_t oracle_pcg_next(or_pcg* r)
{
	uint64_t old = r->state;
	r->state = old * PCG_MULT + r->inc;
	uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
	uint32_t rot = (uint32_t)(old >> 59u);
	return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

void oracle_pcg_seed(or_pcg* r, uint64_t initstate, uint64_t initseq)
{
	r->state = 0u;
	r->inc = (initseq << 1u) | 1u;
	oracle_pcg_next(r);
	r->state += initstate;
	oracle_pcg_next(r);
}

float oracle_pcg_uniform(or_pcg* r) { return (float)(oracle_pcg_next(r) >> 8) * 0x1.0p-24f; }

void oracle_pixel_stream(or_pcg* r, uint64_t seed, uint32_t frame, uint32_t pixel, uint32_t stage)
{
	uint64_t initstate = seed ^ ((uint64_t)frame * 0x9E3779B97F4A7C15ull);
	uint64_t initseq = ((uint64_t)pixel << 2) | (uint64_t)(stage & 3u);
	oracle_pcg_seed(r, initstate, initseq);
}

void oracle_sincos_2pi(float r, float* s, float* c)
{
	float q = r * 4.0f;            /* exact */
	int k = (int)q;                /* quadrant 0..3 */
	if (k > 3) k = 3;
	if (k < 0) k = 0;
	float f = q - (float)k;        /* exact, in [0, 1) */
	int swap = f > 0.5f;
	float g = swap ? (1.0f - f) : f; /* exact, in [0, 0.5] */
	float x = g * 0x1.921fb6p+0f;  /* g * pi/2, in [0, pi/4] */
	float x2 = x * x;
	float sp = x * (1.0f + x2 * (-0x1.555556p-3f + x2 * (0x1.111112p-7f + x2 * (-0x1.a01a02p-13f + x2 * 0x1.71de3ap-19f))));
	float cp = 1.0f + x2 * (-0x1.0p-1f + x2 * (0x1.555556p-5f + x2 * (-0x1.6c16c2p-10f + x2 * (0x1.a01a02p-16f - x2 * 0x1.27e4fcp-22f))));
	float sq = swap ? cp : sp;     /* sin(f * pi/2) */
	float cq = swap ? sp : cp;     /* cos(f * pi/2) */
	switch (k) {
	case 0: *s = sq; *c = cq; break;
	case 1: *s = cq; *c = -sq; break;
	case 2: *s = -sq; *c = -cq; break;
	default: *s = -cq; *c = sq; break;
	}
}

/* ---------------------------------------------------------------------------------------------
 * Shading (CudaPbr.cuh:26-111)
 * ------------------------------------------------------------------------------------------- */

#define OR_PI_D 3.141592653589793 /* CUDART_PI (double) */
#define OR_PI_F 3.14159274f       /* float(CUDART_PI) */

static float ggx(float nDotH, float a)
{
	float a2 = a * a;
	float base = nDotH * nDotH * (a2 - 1.0f) + 1.0f;
	float div = (float)(OR_PI_D * (double)(base * base)); /* double constant, stored to float */
	return a2 / div;
}

static float geometric_schlick(float nDotL, float nDotV, float k)
{
	float g1 = nDotL / (nDotL * (1.0f - k) + k);
	float g2 = nDotV / (nDotV * (1.0f - k) + k);
	return g1 * g2;
}

static inline float cuda_clamp(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
/* lerp of CudaDeviceHelpers.cuh:24-27: fma(t, v1, fma(-t, v0, v0)). */
static inline float cuda_lerp(float v0, float v1, float t) { return fmaf(t, v1, fmaf(-t, v0, v0)); }

void oracle_shade(const float pp[3], const float nn[3], const float vv[3], const float albedo[3], float roughness,
                  float metallic, const float ll[3], float toLightDist, const float strength[3], float range,
                  float out[3])
{
	(void)pp;
	out[0] = out[1] = out[2] = 0.0f;
	if (toLightDist > range) return;
	v3 n = ld3(nn), v = ld3(vv), l = ld3(ll), alb = ld3(albedo);
	v3 h = normalize3(add(l, v));
	float nDotL = dot(n, l);
	if (nDotL <= 0.0f) return;
	float nDotV = fmaxf(0.001f, dot(n, v));
	v3 diffuse = divs(alb, OR_PI_F);
	float nDotH = fmaxf(0.0f, dot(n, h));
	float ctD = ggx(nDotH, roughness * roughness);
	float rp1 = roughness + 1.0f;
	float k = (rp1 * rp1) / 8.0f;
	float ctG = geometric_schlick(nDotL, nDotV, k);
	v3 f0 = mk(cuda_lerp(0.04f, alb.x, metallic), cuda_lerp(0.04f, alb.y, metallic), cuda_lerp(0.04f, alb.z, metallic));
	float om = 1.0f - nDotV;
	float om2 = om * om;
	float p5 = cuda_clamp(om2 * om2 * om, 0.0f, 1.0f);
	v3 ctF = add(f0, muls(sub(mk(1.0f, 1.0f, 1.0f), f0), p5));
	v3 specular = divs(muls(muls(ctF, ctD), ctG), 4.0f * nDotL * nDotV);
	v3 ks = ctF;
	v3 kd = muls(sub(mk(1.0f, 1.0f, 1.0f), ks), 1.0f - metallic);
	v3 shaded = muls(mulv(add(mulv(kd, diffuse), specular), ld3(strength)), nDotL);
	if (!isfinite(shaded.x) || !isfinite(shaded.y) || !isfinite(shaded.z)) shaded = mk(0.0f, 0.0f, 0.0f);
	out[0] = shaded.x; out[1] = shaded.y; out[2] = shaded.z;
}

float oracle_falloff(float toLightDist, float range)
{
	float x = toLightDist / range;
	float x2 = x * x;
	float c = cuda_clamp(1.0f - x2 * x2, 0.0f, 1.0f);
	float num = c * c;
	float den = (float)((double)(toLightDist * toLightDist) + 1.0); /* `+ 1.0` is a double literal */
	return num / den;
}

/* hemisphereToWorld (MaterialKernel.cu:206-218) given cos/sin of phi. */
static v3 hemisphere_to_world(float cphi, float sphi, float cosTheta, float sinTheta, v3 normal)
{
	float hx = sinTheta * cphi, hy = sinTheta * sphi, hz = cosTheta;
	v3 upVector = fabsf(normal.z) < 0.999f ? mk(0.0f, 0.0f, 1.0f) : mk(1.0f, 0.0f, 0.0f);
	v3 u = normalize3(cross(upVector, normal));
	v3 v = cross(normal, u);
	return add(add(muls(u, hx), muls(v, hy)), muls(normal, hz));
}

void oracle_sample_lambert(float r1, float r2, const float nn[3], float out[3])
{
	float s, c;
	oracle_sincos_2pi(r1, &s, &c);
	float sinTheta = sqrtf(r2);
	float cosTheta = sqrtf(1.0f - r2);
	v3 d = hemisphere_to_world(c, s, cosTheta, sinTheta, ld3(nn));
	out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

static v3 sample_ggx(float r1, float r2, float a, v3 reflection, v3 surfaceNormal)
{
	float s, c;
	oracle_sincos_2pi(r1, &s, &c);
	float cosTheta = sqrtf((1.0f - r2) / (1.0f + (a * a - 1.0f) * r2));
	float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
	v3 vec = hemisphere_to_world(c, s, cosTheta, sinTheta, reflection);
	float nDotV = dot(vec, surfaceNormal);
	float off = -stdmin(0.0f, nDotV);
	return normalize3(add(vec, muls(surfaceNormal, off)));
}

/* reflect (CudaDeviceHelpers.cuh:44-47): in - 2 dot(n, in) n */
static v3 reflect3(v3 in, v3 n) { return sub(in, muls(n, 2.0f * dot(n, in))); }

/* The GGX branch of the bounce (MaterialKernel.cu:293-299): a = roughness^2 around reflect(fromCamera, n). */
static v3 bounce_ggx(float r1, float r2, float roughness, v3 fromCamera, v3 normal)
{
	return sample_ggx(r1, r2, roughness * roughness, reflect3(fromCamera, normal), normal);
}

void oracle_sample_ggx_bounce(float r1, float r2, float roughness, const float fromCamera[3], const float nn[3],
                              float out[3])
{
	v3 d = bounce_ggx(r1, r2, roughness, ld3(fromCamera), ld3(nn));
	out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

/* ---------------------------------------------------------------------------------------------
 * Wavefront frame
 * ------------------------------------------------------------------------------------------- */

/* Surface values at a hit: albedo rgb + alpha, roughness, metallic (constants or texels). */
typedef struct { float albedo[4]; float roughness; float metallic; } or_surface;
typedef struct { v3 pos, normal; or_surface surf; } hit_info;

uint32_t oracle_texel_coord(float c, int32_t n)
{
	float f = c - floorf(c);
	if (!(f >= 0.0f)) return 0u;
	uint32_t i = (uint32_t)(f * (float)n);
	return i >= (uint32_t)n ? 0u : i;
}

void oracle_srgb_table(float out[256])
{
	for (int b = 0; b < 256; b++) out[b] = (float)pow((double)((float)b / 255.0f), (double)2.2f);
}

static const uint8_t* texel_at(const or_texture* t, float u, float v)
{
	uint32_t i = oracle_texel_coord(u, t->width), jj = oracle_texel_coord(v, t->height);
	return t->data + (size_t)jj * t->pitch + (size_t)i * t->bytesPerPixel;
}

/* retrieveTriData (InterpretRayHitKernel.cu:13-37): position and interpolated normal at a hit. */
static void retrieve_tri_data(const or_tri_data* d, const or_ray* r, const or_hit* h, v3* pos, v3* normal)
{
	*pos = add(ld3(r->o), muls(ld3(r->d), h->t));
	v3 n0 = ld3(d->n0), n1 = ld3(d->n1), n2 = ld3(d->n2);
	*normal = normalize3(add(add(n0, muls(sub(n1, n0), h->u)), muls(sub(n2, n0), h->v)));
}

/* uv at a hit: uv0 + (uv1 - uv0) u + (uv2 - uv0) v, left to right */
static void hit_uv(const or_tri_data* d, const or_hit* h, float* tu, float* tv)
{
	*tu = (d->uv0[0] + (d->uv1[0] - d->uv0[0]) * h->u) + (d->uv2[0] - d->uv0[0]) * h->v;
	*tv = (d->uv0[1] + (d->uv1[1] - d->uv0[1]) * h->u) + (d->uv2[1] - d->uv0[1]) * h->v;
}

void oracle_retrieve_tri_data(uint32_t n, const or_tri_data* datas, const or_ray* rays, const or_hit* hits, float* out,
                              uint32_t* materialIndex)
{
	for (uint32_t i = 0; i < n; i++) {
		v3 pos, normal;
		retrieve_tri_data(&datas[i], &rays[i], &hits[i], &pos, &normal);
		float* o = out + 8 * (size_t)i;
		o[0] = pos.x; o[1] = pos.y; o[2] = pos.z;
		o[3] = normal.x; o[4] = normal.y; o[5] = normal.z;
		hit_uv(&datas[i], &hits[i], &o[6], &o[7]);
		materialIndex[i] = datas[i].materialIndex;
	}
}

static hit_info interpret(const or_tri_data* datas, const or_frame_params* fp, const float* srgb, const or_ray* r,
                          const or_hit* h)
{
	/* retrieveTriData + material lookup (InterpretRayHitKernel.cu:13-37, 60-121) */
	hit_info hi;
	const or_tri_data* d = &datas[h->tri];
	retrieve_tri_data(d, r, h, &hi.pos, &hi.normal);
	const or_material* m = &fp->materials[d->materialIndex];
	for (int k = 0; k < 4; k++) hi.surf.albedo[k] = m->albedo[k];
	hi.surf.roughness = m->roughness;
	hi.surf.metallic = m->metallic;
	if (m->texIndex[0] >= 0 || m->texIndex[1] >= 0 || m->texIndex[2] >= 0) {
		float tu, tv;
		hit_uv(d, h, &tu, &tv);
		if (m->texIndex[0] >= 0) {
			const uint8_t* c = texel_at(&fp->textures[m->texIndex[0]], tu, tv);
			for (int k = 0; k < 3; k++) hi.surf.albedo[k] = srgb[c[k]];
			hi.surf.albedo[3] = (float)c[3] / 255.0f;
		}
		if (m->texIndex[1] >= 0) hi.surf.roughness = (float)*texel_at(&fp->textures[m->texIndex[1]], tu, tv) / 255.0f;
		if (m->texIndex[2] >= 0) hi.surf.metallic = (float)*texel_at(&fp->textures[m->texIndex[2]], tu, tv) / 255.0f;
	}
	return hi;
}

/* shadeHit (MaterialKernel.cu:49-112) for one light: contribution and, when cast, the shadow ray. The
 * two uniform numbers of the soft-shadow offset come from `rng`, or from fixedR[0..1] when rng is NULL. */
static int shade_light(const or_light* light, v3 mask, v3 normal, v3 toCamera, v3 pos, const or_surface* m,
                       or_pcg* rng, const float* fixedR, float contrib[3], or_ray* shadowRay)
{
	v3 lp = ld3(light->pos);
	v3 toLight = sub(lp, pos);
	float toLightDist = length3(toLight);
	v3 l = divs(toLight, toLightDist);
	float falloff = oracle_falloff(toLightDist, light->range);
	float sh[3];
	float pa[3] = {pos.x, pos.y, pos.z}, na[3] = {normal.x, normal.y, normal.z};
	float va[3] = {toCamera.x, toCamera.y, toCamera.z}, la[3] = {l.x, l.y, l.z};
	oracle_shade(pa, na, va, m->albedo, m->roughness, m->metallic, la, toLightDist, light->strength, light->range, sh);
	v3 shading = mulv(muls(mask, falloff), ld3(sh));
	contrib[0] = shading.x; contrib[1] = shading.y; contrib[2] = shading.z;
	const float EPSILON = 0.0001f;
	int contributes = shading.x > EPSILON || shading.y > EPSILON || shading.z > EPSILON;
	if (!(light->staticShadows && contributes)) return 0;
	v3 circleU = fabsf(normal.z) > 0.01f ? normalize3(mk(0.0f, -normal.z, normal.y))
	                                     : normalize3(mk(-normal.y, normal.x, 0.0f));
	v3 circleV = cross(circleU, l);
	float r1 = rng ? oracle_pcg_uniform(rng) : fixedR[0];
	float r2 = rng ? oracle_pcg_uniform(rng) : fixedR[1];
	float centerDistance = light->radius * (2.0f * r2 - 1.0f);
	float s, c;
	oracle_sincos_2pi(r1, &s, &c);
	v3 offset = add(muls(muls(circleU, c), centerDistance), muls(muls(circleV, s), centerDistance));
	v3 diff = sub(add(lp, offset), pos);
	v3 dir = normalize3(diff);
	shadowRay->o[0] = pos.x; shadowRay->o[1] = pos.y; shadowRay->o[2] = pos.z;
	shadowRay->d[0] = dir.x; shadowRay->d[1] = dir.y; shadowRay->d[2] = dir.z;
	shadowRay->tmin = 0.001f;
	shadowRay->tmax = length3(diff);
	return 1;
}

int oracle_shade_hit(const or_light* light, const float mask[3], const float normal[3], const float toCamera[3],
                     const float pos[3], const float albedo[3], float metallic, float roughness, const float r12[2],
                     float contrib[3], or_ray* shadowRay)
{
	or_surface m;
	m.albedo[0] = albedo[0]; m.albedo[1] = albedo[1]; m.albedo[2] = albedo[2]; m.albedo[3] = 1.0f;
	m.roughness = roughness;
	m.metallic = metallic;
	return shade_light(light, ld3(mask), ld3(normal), ld3(toCamera), ld3(pos), &m, NULL, r12, contrib, shadowRay);
}

typedef struct {
	const or_node* nodes; const or_tri* tris; const or_tri_data* datas; const or_frame_params* fp;
	const or_hit* primaryHits; float* color; float* roughnessOut;
	float srgb[256];
	atomic_uint next; atomic_ullong counts[4]; atomic_ullong work[8]; atomic_int overflows;
	atomic_uint dumpNext[4];
} frame_job;

static int cast1(frame_job* j, const or_ray* r, or_hit* h, int stage)
{
	if (j->fp->dump[stage]) {
		uint32_t k = atomic_fetch_add(&j->dumpNext[stage], 1u);
		if (k < j->fp->dumpCapacity[stage]) j->fp->dump[stage][k] = *r;
	}
	uint32_t nv = 0, nt = 0;
	int rc = oracle_cast_ray(j->nodes, j->tris, r, OR_MODE_REFERENCE_GPU, h, &nv, &nt);
	atomic_fetch_add(&j->work[2 * stage], (unsigned long long)nv);
	atomic_fetch_add(&j->work[2 * stage + 1], (unsigned long long)nt);
	return rc;
}

/* uv of the camera ray through d (a point minus the camera origin, or a direction); 0 behind the camera */
static int project_uv(const or_camera* c, v3 d, float* u, float* v)
{
	v3 dir = ld3(c->dir), dX = ld3(c->dX), dY = ld3(c->dY);
	float z = dot(d, dir);
	if (!(z > 0.0f)) return 0;
	float cx = dot(d, dX) / (dot(dX, dX) * z);
	float cy = dot(d, dY) / (dot(dY, dY) * z);
	*u = (cx + 1.0f) * 0.5f;
	*v = (cy + 1.0f) * 0.5f;
	return 1;
}

static void pixel_velocity(const or_frame_params* fp, int hit, v3 pos, v3 dir, float* out)
{
	float u0, v0, u1, v1;
	v3 d0 = hit ? sub(pos, ld3(fp->cam.origin)) : dir, d1 = hit ? sub(pos, ld3(fp->prevCam.origin)) : dir;
	if (project_uv(&fp->cam, d0, &u0, &v0) && project_uv(&fp->prevCam, d1, &u1, &v1)) {
		out[0] = u0 - u1;
		out[1] = v0 - v1;
	} else {
		out[0] = 2.0f;
		out[1] = 2.0f;
	}
}

static void frame_pixel(frame_job* j, uint32_t x, uint32_t y)
{
	const or_frame_params* fp = j->fp;
	uint32_t pid = y * fp->resX + x;
	float* col = &j->color[4 * (size_t)pid];
	col[0] = col[1] = col[2] = 0.0f; col[3] = 1.0f;
	if (j->roughnessOut) j->roughnessOut[pid] = 0.0f;
	uint64_t counts[4] = {1, 0, 0, 0};

	/* Primary ray (genPrimaryRaysKernel with the jitter offset). */
	or_ray pr;
	v3 d = primary_dir(&fp->cam, (float)x + fp->jitter[0], (float)y + fp->jitter[1], (float)fp->resX, (float)fp->resY);
	pr.o[0] = fp->cam.origin[0]; pr.o[1] = fp->cam.origin[1]; pr.o[2] = fp->cam.origin[2];
	pr.tmin = 0.0001f; pr.d[0] = d.x; pr.d[1] = d.y; pr.d[2] = d.z; pr.tmax = FLT_MAX;
	or_hit ph;
	if (j->primaryHits) ph = j->primaryHits[pid];
	else if (cast1(j, &pr, &ph, 0)) atomic_fetch_add(&j->overflows, 1);
	if (fp->velocity && ph.tri == ~0u) pixel_velocity(fp, 0, mk(0.0f, 0.0f, 0.0f), ld3(pr.d), &fp->velocity[2 * pid]);
	if (ph.tri == ~0u) goto done;
	{
		hit_info hi = interpret(j->datas, fp, j->srgb, &pr, &ph);
		if (fp->velocity) pixel_velocity(fp, 1, hi.pos, ld3(pr.d), &fp->velocity[2 * pid]);
		if (j->roughnessOut) j->roughnessOut[pid] = hi.surf.roughness;
		or_pcg rng;
		oracle_pixel_stream(&rng, fp->seed, fp->frame, pid, 0);
		v3 toCamera = normalize3(sub(ld3(fp->camPos), hi.pos));
		v3 accum = mk(0.0f, 0.0f, 0.0f);
		for (uint32_t li = 0; li < fp->numLights; li++) {
			float c[3];
			or_ray sr;
			int inLight = 1;
			if (shade_light(&fp->lights[li], mk(1.0f, 1.0f, 1.0f), hi.normal, toCamera, hi.pos, &hi.surf, &rng, NULL, c, &sr)) {
				or_hit sh;
				counts[1]++;
				if (cast1(j, &sr, &sh, 1)) atomic_fetch_add(&j->overflows, 1);
				inLight = sh.tri == ~0u;
			}
			if (inLight) accum = add(accum, ld3(c));
		}

		/* Bounce (createSecondaryRaysKernel, MaterialKernel.cu:251-312, full resolution). */
		float r1 = oracle_pcg_uniform(&rng);
		float r2 = oracle_pcg_uniform(&rng);
		v3 throughput = mk(1.0f, 1.0f, 1.0f);
		or_ray br;
		br.tmin = 0.001f;
		br.tmax = FLT_MAX;
		v3 bdir;
		const or_surface* m = &hi.surf;
		v3 alb = ld3(m->albedo);
		v3 fromCamera = normalize3(sub(hi.pos, ld3(fp->camPos)));
		if (m->albedo[3] > 0.5f) {
			float r3 = oracle_pcg_uniform(&rng);
			throughput = mulv(throughput, alb);
			if (r3 < m->roughness) {
				float na[3] = {hi.normal.x, hi.normal.y, hi.normal.z}, o3[3];
				oracle_sample_lambert(r1, r2, na, o3);
				bdir = ld3(o3);
			} else {
				bdir = bounce_ggx(r1, r2, m->roughness, fromCamera, hi.normal);
			}
			throughput = muls(throughput, 0.6f);
		} else {
			bdir = normalize3(add(muls(fromCamera, 0.8f), muls(mk(-hi.normal.x, -hi.normal.y, -hi.normal.z), 0.2f)));
			br.tmin = 0.2f;
		}
		br.o[0] = hi.pos.x; br.o[1] = hi.pos.y; br.o[2] = hi.pos.z;
		br.d[0] = bdir.x; br.d[1] = bdir.y; br.d[2] = bdir.z;
		counts[2]++;
		or_hit bh;
		if (cast1(j, &br, &bh, 2)) atomic_fetch_add(&j->overflows, 1);
		if (bh.tri != ~0u) {
			hit_info bi = interpret(j->datas, fp, j->srgb, &br, &bh);
			or_pcg rng2;
			oracle_pixel_stream(&rng2, fp->seed, fp->frame, pid, 1);
			v3 toCam2 = mk(-br.d[0], -br.d[1], -br.d[2]);
			for (uint32_t li = 0; li < fp->numLights; li++) {
				float c[3];
				or_ray sr;
				int inLight = 1;
				if (shade_light(&fp->lights[li], throughput, bi.normal, toCam2, bi.pos, &bi.surf, &rng2, NULL, c, &sr)) {
					or_hit sh;
					counts[3]++;
					if (cast1(j, &sr, &sh, 3)) atomic_fetch_add(&j->overflows, 1);
					inLight = sh.tri == ~0u;
				}
				if (inLight) accum = add(accum, ld3(c));
			}
		}
		col[0] = accum.x; col[1] = accum.y; col[2] = accum.z;
	}
done:
	for (int i = 0; i < 4; i++) atomic_fetch_add(&j->counts[i], counts[i]);
}

static void* frame_worker(void* arg)
{
	frame_job* j = (frame_job*)arg;
	uint32_t W = j->fp->resX, H = j->fp->resY;
	uint32_t end = j->fp->rowEnd && j->fp->rowEnd < H ? j->fp->rowEnd : H;
	for (;;) {
		uint32_t row = j->fp->rowBegin + atomic_fetch_add(&j->next, 1u);
		if (row >= end) break;
		for (uint32_t x = 0; x < W; x++) frame_pixel(j, x, row);
	}
	return NULL;
}

int oracle_render_frame(const or_node* nodes, const or_tri* tris, const or_tri_data* datas,
                        const or_frame_params* fp, const or_hit* primaryHits, float* color, float* roughnessOut,
                        uint64_t* rayCounts, uint64_t* workSums, int threads)
{
	frame_job j;
	memset(&j, 0, sizeof(j));
	j.nodes = nodes; j.tris = tris; j.datas = datas; j.fp = fp; j.primaryHits = primaryHits;
	j.color = color; j.roughnessOut = roughnessOut;
	oracle_srgb_table(j.srgb);
	atomic_init(&j.next, 0u);
	for (int i = 0; i < 4; i++) atomic_init(&j.counts[i], 0ull);
	for (int i = 0; i < 8; i++) atomic_init(&j.work[i], 0ull);
	for (int i = 0; i < 4; i++) atomic_init(&j.dumpNext[i], 0u);
	atomic_init(&j.overflows, 0);
	if (threads < 1) threads = 1;
	pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
	int started = 0;
	for (int t = 0; t < threads; t++)
		if (pthread_create(&th[t], NULL, frame_worker, &j) == 0) started++;
		else break;
	if (started == 0) frame_worker(&j);
	for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
	free(th);
	if (rayCounts)
		for (int i = 0; i < 4; i++) rayCounts[i] = atomic_load(&j.counts[i]);
	if (workSums)
		for (int i = 0; i < 8; i++) workSums[i] = atomic_load(&j.work[i]);
	if (fp->dumpCount)
		for (int i = 0; i < 4; i++) fp->dumpCount[i] = atomic_load(&j.dumpNext[i]);
	return atomic_load(&j.overflows);
}

/* ---------------------------------------------------------------------------------------------
 * TAA (taa.frag:25-71), with the history fetched in pixel space
 * ------------------------------------------------------------------------------------------- */

static inline float glsl_mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }

/* GL_LINEAR, clamp to edge, at pixel-space position (px, py) measured from the texel grid origin
 * (texel centres at integer + 0.5). Channel count `ch`. */
static void bilinear(const float* tex, uint32_t W, uint32_t H, int ch, float px, float py, float* out)
{
	float fx = px - 0.5f, fy = py - 0.5f;
	float x0f = floorf(fx), y0f = floorf(fy);
	float ax = fx - x0f, ay = fy - y0f;
	long x0 = (long)x0f, y0 = (long)y0f, x1 = x0 + 1, y1 = y0 + 1;
	if (x0 < 0) x0 = 0; if (x0 > (long)W - 1) x0 = (long)W - 1;
	if (x1 < 0) x1 = 0; if (x1 > (long)W - 1) x1 = (long)W - 1;
	if (y0 < 0) y0 = 0; if (y0 > (long)H - 1) y0 = (long)H - 1;
	if (y1 < 0) y1 = 0; if (y1 > (long)H - 1) y1 = (long)H - 1;
	for (int c = 0; c < ch; c++) {
		float t00 = tex[((size_t)y0 * W + (size_t)x0) * ch + c], t10 = tex[((size_t)y0 * W + (size_t)x1) * ch + c];
		float t01 = tex[((size_t)y1 * W + (size_t)x0) * ch + c], t11 = tex[((size_t)y1 * W + (size_t)x1) * ch + c];
		float top = glsl_mix(t00, t10, ax), bot = glsl_mix(t01, t11, ax);
		out[c] = glsl_mix(top, bot, ay);
	}
}

void oracle_taa(uint32_t W, uint32_t H, const float* cur, const float* hist, const float* velocity,
                const float* prevVelocity, const float* roughness, float* outColor, float* outHist)
{
	for (uint32_t y = 0; y < H; y++)
		for (uint32_t x = 0; x < W; x++) {
			size_t p = (size_t)y * W + x;
			const float* c = &cur[4 * p];
			float vx = velocity ? velocity[2 * p] : 0.0f, vy = velocity ? velocity[2 * p + 1] : 0.0f;
			/* historyCoord = uv - velocity, in pixels: (x + 0.5) - vx * W */
			float hx = ((float)x + 0.5f) - vx * (float)W;
			float hy = ((float)y + 0.5f) - vy * (float)H;
			float* oh = &outHist[4 * p];
			float* oc = &outColor[4 * p];
			if (hx < 0.0f || hx > (float)W || hy < 0.0f || hy > (float)H) {
				oh[0] = c[0]; oh[1] = c[1]; oh[2] = c[2]; oh[3] = 1.0f;
				oc[0] = c[0]; oc[1] = c[1]; oc[2] = c[2]; oc[3] = 1.0f;
				continue;
			}
			float hv[2] = {0.0f, 0.0f};
			if (prevVelocity) {
				if (vx == 0.0f && vy == 0.0f) { hv[0] = prevVelocity[2 * p]; hv[1] = prevVelocity[2 * p + 1]; }
				else bilinear(prevVelocity, W, H, 2, hx, hy, hv);
			}
			float pvx = (float)W * vx, pvy = (float)H * vy;
			float hpx = (float)W * hv[0], hpy = (float)H * hv[1];
			float lp = sqrtf(pvx * pvx + pvy * pvy), lh = sqrtf(hpx * hpx + hpy * hpy);
			float velocityDistrust = fminf(1.0f, 1.2f * sqrtf(fabsf(lp - lh)));
			float roughnessDistrust = glsl_mix(3.0f, 1.0f, roughness ? roughness[p] : 0.0f);
			float trust = cuda_clamp(1.0f - roughnessDistrust * velocityDistrust, 0.0f, 1.0f);
			float h4[4];
			if (vx == 0.0f && vy == 0.0f) memcpy(h4, &hist[4 * p], 16);
			else bilinear(hist, W, H, 4, hx, hy, h4);
			float newSamples = h4[3] * trust + 1.0f;
			float blend = 1.0f - 1.0f / newSamples;
			for (int k = 0; k < 3; k++) {
				oh[k] = glsl_mix(c[k], h4[k], blend);
				oc[k] = oh[k];
			}
			oh[3] = newSamples;
			oc[3] = 1.0f;
		}
}

void oracle_halton_jitter(uint32_t i, float out[2])
{
	/* Radical inverse in bases 2 and 3 of i + 1, rounded to float, matching the 16-entry table
	 * HALTON_SEQ of GameScreen.cpp:21-39 (entries 1..16 of the sequence). */
	uint32_t k = (i % 16u) + 1u;
	double f = 1.0, r = 0.0;
	uint32_t n = k;
	while (n) { f /= 2.0; r += f * (double)(n % 2u); n /= 2u; }
	double f3 = 1.0, r3 = 0.0;
	n = k;
	while (n) { f3 /= 3.0; r3 += f3 * (double)(n % 3u); n /= 3u; }
	out[0] = (float)r - 0.5f;
	out[1] = (float)r3 - 0.5f;
}

/* ---------------------------------------------------------------------------------------------
 * Display post-process (gamma_correction.frag:20-74)
 * ------------------------------------------------------------------------------------------- */

static float u2_tonemap(float x)
{
	const float A = 0.25f, B = 0.25f, C = 0.105f, D = 0.20f, E = 0.025f, F = 0.25f;
	return (x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F) - E / F;
}

void oracle_scale(uint32_t srcW, uint32_t srcH, const float* src, uint32_t vpW, uint32_t vpH, uint32_t dstW,
                  uint32_t dstH, float* dst)
{
	/* scaling.frag:19-35 */
	const float dw = (float)dstW, dh = (float)dstH, sw = (float)srcW, sh = (float)srcH;
	const float ox = (1.0f / dw) * 0.25f, oy = (1.0f / dh) * 0.25f;
	const float sx[4] = {-ox, ox, -ox, ox}, sy[4] = {-oy, -oy, oy, oy};
	for (uint32_t y = 0; y < dstH; y++)
		for (uint32_t x = 0; x < dstW; x++) {
			float u = ((float)x + 0.5f) / dw, v = ((float)y + 0.5f) / dh;
			float cx = (u * (float)vpW) / sw, cy = (v * (float)vpH) / sh;
			float acc[3] = {0.0f, 0.0f, 0.0f};
			for (int k = 0; k < 4; k++) {
				float t[4];
				bilinear(src, srcW, srcH, 4, (cx + sx[k]) * sw, (cy + sy[k]) * sh, t);
				for (int c = 0; c < 3; c++) acc[c] = k == 0 ? t[c] : acc[c] + t[c];
			}
			float* o = &dst[4 * ((size_t)y * dstW + x)];
			for (int c = 0; c < 3; c++) o[c] = acc[c] / 4.0f;
			o[3] = 1.0f;
		}
}

void oracle_postprocess(uint32_t n, const float* linear, float gamma, float* display)
{
	const float W = 11.2f, BLACK_CRUSH = 0.0015f, exposureBias = 2.0f;
	float invGamma = 1.0f / gamma;
	float white = u2_tonemap(W);
	for (uint32_t i = 0; i < n; i++) {
		for (int k = 0; k < 3; k++) {
			float x = exposureBias * fmaxf(0.0f, linear[4 * (size_t)i + k] - BLACK_CRUSH);
			display[4 * (size_t)i + k] = powf(u2_tonemap(x) / white, invGamma);
		}
		display[4 * (size_t)i + 3] = linear[4 * (size_t)i + 3];
	}
}
