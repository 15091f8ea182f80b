// ORCA linear programs on the device (warp-uniform; LP3 builds its projected
// lines lane-parallel).  Restates linearProgram1/2/3 of the reference's
// RVO2-derived solver, src/3rd-party/ORCA/ORCASolver.cpp:173-326.
#pragma once
#include "devmath.cuh"

namespace umans {

// ORCA (ORCASolver.cpp:61-326, CostFunctions/ORCA.cpp:26-95)
// lines are float4 (point.x, point.y, direction.x, direction.y)
// ------------------------------------------------------------------------
__device__ __forceinline__ float det2(float2 a, float2 b) { return a.x * b.y - a.y * b.x; }
__device__ __forceinline__ float2 lp_point(float4 l) { return V(l.x, l.y); }
__device__ __forceinline__ float2 lp_dir(float4 l) { return V(l.z, l.w); }

// order-preserving unsigned keys of finite floats (for warp min / max by
// redux.sync)
__device__ __forceinline__ unsigned lp_key(float f)
{
	const unsigned u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float lp_val(unsigned k)
{
	return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// linearProgram1 (ORCASolver.cpp:173-226), the warp splitting the earlier
// lines.  tl only grows and tr only shrinks along the reference's loop, so
// its early exits (a parallel line excluding the whole line, or tl > tr at
// some prefix) give the same answer as testing the whole set at once; the
// bounds are the maximum / minimum of the same values.
static __device__ bool lp1(const float4* L, int lineNo, float radius, float2 opt, bool dirOpt, float2* res, int lane)
{
	const float4 ln = L[lineNo];
	const float2 P = lp_point(ln), D = lp_dir(ln);
	const float dp = vdot(P, D);
	const float disc = dp * dp + radius * radius - vsq(P);
	if (disc < 0.0f) return false;
	const float sd = sqrtf(disc);
	float tl = -dp - sd, tr = -dp + sd;
	bool bad = false;
	for (int i = lane; i < lineNo; i += 32) {
		const float4 li = L[i];
		const float den = det2(D, lp_dir(li));
		const float num = det2(lp_dir(li), vsub(P, lp_point(li)));
		if (fabsf(den) <= 0.00001f) {
			if (num < 0.0f) bad = true;
			continue;
		}
		const float t = num / den;
		if (den >= 0.0f) tr = fminr(tr, t);
		else tl = fmaxr(tl, t);
	}
	// one warp reduction each, the same value on every lane (of equal values
	// of different zero sign the minimum takes -0, the maximum +0; either is
	// exact for the uses below)
	tr = lp_val(__reduce_min_sync(0xffffffffu, lp_key(tr)));
	tl = lp_val(__reduce_max_sync(0xffffffffu, lp_key(tl)));
	if (__any_sync(0xffffffffu, bad) || tl > tr) return false;
	if (dirOpt) {
		if (vdot(opt, D) > 0.0f) *res = vadd(P, vmul(D, tr));
		else *res = vadd(P, vmul(D, tl));
	} else {
		const float t = vdot(D, vsub(opt, P));
		if (t < tl) *res = vadd(P, vmul(D, tl));
		else if (t > tr) *res = vadd(P, vmul(D, tr));
		else *res = vadd(P, vmul(D, t));
	}
	return true;
}

// linearProgram2 (ORCASolver.cpp:228-267): the warp looks for the next line
// the current result violates 32 lines at a time; lines it satisfies leave
// the reference's loop unchanged.
static __device__ int lp2(const float4* L, int n, float radius, float2 opt, bool dirOpt, float2* res, int lane)
{
	if (dirOpt) *res = vmul(opt, radius);
	else if (vsq(opt) > radius * radius) *res = vmul(vnorm(opt), radius);
	else *res = opt;
	int i = 0;
	while (i < n) {
		int viol = n;
		for (int base = i; base < n; base += 32) {
			const int j = base + lane;
			bool v = false;
			if (j < n) {
				const float4 lj = L[j];
				v = det2(lp_dir(lj), vsub(lp_point(lj), *res)) > 0.0f;
			}
			const unsigned m = __ballot_sync(0xffffffffu, v);
			if (m) { viol = base + __ffs(m) - 1; break; }
		}
		if (viol == n) return n;
		const float2 tmp = *res;
		if (!lp1(L, viol, radius, opt, dirOpt, res, lane)) { *res = tmp; return viol; }
		i = viol + 1;
	}
	return n;
}

static __device__ void lp3(const float4* L, int n, int begin, float radius, float2* res, float4* proj, int lane)
{
	float distance = 0.0f;
	for (int i = begin; i < n; ++i) {
		const float4 li = L[i];
		const float2 Pi = lp_point(li), Di = lp_dir(li);
		if (det2(Di, vsub(Pi, *res)) > distance) {
			// projected lines, built lane-parallel and compacted in order
			int np = 0;
			for (int base = 0; base < i; base += 32) {
				const int j = base + lane;
				bool keep = false;
				float4 out = make_float4(0, 0, 0, 0);
				if (j < i) {
					const float4 lj = L[j];
					const float2 Pj = lp_point(lj), Dj = lp_dir(lj);
					const float determinant = det2(Di, Dj);
					float2 pt;
					keep = true;
					if (fabsf(determinant) <= 0.00001f) {
						if (vdot(Di, Dj) > 0.0f) keep = false;
						else pt = vmul(vadd(Pi, Pj), 0.5f);
					} else {
						pt = vadd(Pi, vmul(Di, det2(Dj, vsub(Pi, Pj)) / determinant));
					}
					if (keep) {
						const float2 d = vnorm(vsub(Dj, Di));
						out = make_float4(pt.x, pt.y, d.x, d.y);
					}
				}
				const unsigned m = __ballot_sync(0xffffffffu, keep);
				if (keep) proj[np + __popc(m & ((1u << lane) - 1u))] = out;
				np += __popc(m);
			}
			__syncwarp();
			const float2 tmp = *res;
			if (lp2(proj, np, radius, V(-Di.y, Di.x), true, res, lane) < np) *res = tmp;
			distance = det2(Di, vsub(Pi, *res));
			__syncwarp();
		}
	}
}

}  // namespace umans
