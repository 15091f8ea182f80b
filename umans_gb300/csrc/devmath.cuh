// Device restatement of the reference's 2-D float math.
//
// Vector2D (src/Engine/tools/vector2D.h) computes in float, one rounding per
// operation, with `v / s` implemented as `(1/s) * v` (vector2D.h:132-135).
// These helpers keep that operation order.  The translation units that
// include this header are compiled with -fmad=false so that nvcc never fuses
// a*b+c into an FMA: the reference's CPU build rounds each product.
//
// FP64 islands: the reference promotes to double in angle()/cosAngle()
// (vector2D.h:172-195), rotateCounterClockwise (:166-170) and pow(x, 2).
// Double throughput on GB300 is ~1/64 of float, so:
//   * cosAngle = (float)(dot / (double)len): a single double division of two
//     float operands rounded to float equals the float division (double
//     rounding is innocuous for p_double >= 2 p_float + 2), so it is computed
//     in float;
//   * comparisons of angle() against a threshold use a float guard band and
//     fall back to the exact double computation only within 1e-6 of it.
#pragma once
#include <cfloat>
#include <cstdint>

#include "refmath.hpp"

namespace umans {

#define UD __device__ __forceinline__

// The host C library's sinf/cosf (refmath.hpp): exception tables of the
// device, set once per device by the engine before the first step that needs
// them.
static __constant__ SinCosExceptions c_sincos;
UD void host_sincosf(float x, float* s, float* c) { ref_sincosf(c_sincos, x, s, c); }
UD float host_sinf(float x) { return ref_sinf(c_sincos, x); }

constexpr float MAXF = FLT_MAX;
constexpr double REF_PI = 3.1415926535897;   // vector2D.h:27

UD float2 V(float x, float y) { return make_float2(x, y); }
UD float2 vadd(float2 a, float2 b) { return V(a.x + b.x, a.y + b.y); }
UD float2 vsub(float2 a, float2 b) { return V(a.x - b.x, a.y - b.y); }
UD float2 vmul(float2 a, float s) { return V(a.x * s, a.y * s); }
UD float2 vdiv(float2 a, float s) { float r = 1.0f / s; return V(a.x * r, a.y * r); }
UD float2 vneg(float2 a) { return V(-a.x, -a.y); }
UD float vdot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
UD float vsq(float2 a) { return a.x * a.x + a.y * a.y; }
UD float vmag(float2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
UD bool viszero(float2 a) { return a.x == 0 && a.y == 0; }
UD float2 vnorm(float2 a)
{
	float m = vmag(a);
	if (m > 0) { a.x = a.x / m; a.y = a.y / m; }
	return a;
}
UD float2 vclamp(float2 v, float maxLength)   // clampVector: vector2D.h:241-247
{
	float m = vmag(v);
	if (m <= maxLength) return v;
	return vmul(vnorm(v), maxLength);
}
UD float fminr(float a, float b) { return (b < a) ? b : a; }   // std::min
UD float fmaxr(float a, float b) { return (a < b) ? b : a; }   // std::max

// (float)((double)a * (double)b - (double)c * (double)d).  The products are
// exact in double; their difference D is formed exactly as a float expansion
// (FMA products and TwoSum) and rounded to float.  That equals the
// double-then-float rounding unless D lies within 2^-10 half-ulp of a float
// rounding boundary or the subtraction cancels badly; those rare cases take
// the FP64 path.
UD float prod_diff_d(float a, float b, float c, float d)
{
	const float sh = a * b, sl = fmaf(a, b, -sh);
	const float th = c * d, tl = fmaf(c, d, -th);
	const float ah = sh - th;
	const float bb = ah - sh;
	const float al = (sh - (ah - bb)) + (-th - bb);
	const float lo = (sl - tl) + al;
	const float aah = fabsf(ah);
	if (aah > 0.0f && fabsf(lo) <= 0x1p-20f * aah && fmaxf(fabsf(sh), fabsf(th)) <= 1024.0f * aah) {
		const float rh = ah + lo;
		const float rl = lo - (rh - ah);
		const uint32_t e = __float_as_uint(rh) & 0x7f800000u;
		if (e > (25u << 23) && e < (254u << 23)) {
			const float half_ulp = __uint_as_float(e - (24u << 23));
			if (fabsf(rl) < half_ulp * 0.9990234375f) return rh;
		}
	}
	return (float)__dsub_rn(__dmul_rn((double)a, (double)b), __dmul_rn((double)c, (double)d));
}

// pow(x,2) - pow(y,2) of floats in double, then to float
// (SocialForcesAvoidance.cpp:86)
UD float sq_diff_d(float x, float y) { return prod_diff_d(x, x, y, y); }

// rotateCounterClockwise with cosf/sinf already evaluated (a float pair):
// each component is a double sum of two exact double products rounded to
// float, exactly as vector2D.h:166-170 (c*x - s*y and s*x + c*y = s*x - (-c)*y)
UD float2 vrot_cs(float2 v, float c, float s)
{
	return V(prod_diff_d(c, v.x, s, v.y), prod_diff_d(s, v.x, -c, v.y));
}

// angle(): vector2D.h:172-186, computed exactly in double
UD float vangle_exact(float2 a, float2 b)
{
	const float lf = vmag(a) * vmag(b);
	const double lengths = (double)lf;
	if (lengths == 0) return 0.0f;
	const double frac = __ddiv_rn((double)vdot(a, b), lengths);
	if (frac < -1 || frac > 1) return 0.0f;
	return (float)acos(frac);
}

// cosAngle(): vector2D.h:188-195; float division == (float)(double division)
UD float vcosangle(float2 a, float2 b)
{
	const float lf = vmag(a) * vmag(b);
	if (lf == 0) return 0.0f;
	return vdot(a, b) / lf;
}

// angle(a, b) > thr, with cos_thr = cos(thr) to within 1e-7 and thr below
// 178 degrees.  angle() is never negative and returns 0 for zero-length
// inputs or |frac| > 1.  For nearly opposite vectors (c <= -0.9999) angle()
// is either about 180 degrees (> thr) or, when the double quotient
// frac = dot / lengths falls below -1, exactly 0; with dot and lengths both
// floats, frac < -1 holds exactly when -dot > lengths (two distinct floats
// differ by at least 2^-24 relative, far above the double rounding of the
// quotient), so no double arithmetic is needed there.
UD bool angle_greater(float2 a, float2 b, float thr, float cos_thr)
{
	if (thr < 0) return true;
	const float lf = vmag(a) * vmag(b);
	if (lf == 0) return false;
	const float d = vdot(a, b);
	const float c = d / lf;
	if (c > cos_thr + 1e-6f) return false;                   // clearly smaller (or frac > 1)
	if (c < cos_thr - 1e-6f && c > -0.9999f) return true;    // clearly larger
	if (c <= -0.9999f) return !(-d > lf);
	return vangle_exact(a, b) > thr;
}

// angle(a, b) < thr (same conditions)
UD bool angle_less(float2 a, float2 b, float thr, float cos_thr)
{
	if (thr <= 0) return false;
	const float lf = vmag(a) * vmag(b);
	if (lf == 0) return true;
	const float d = vdot(a, b);
	const float c = d / lf;
	if (c > cos_thr + 1e-6f) return true;
	if (c < cos_thr - 1e-6f && c > -0.9999f) return false;
	if (c <= -0.9999f) return -d > lf;
	return vangle_exact(a, b) < thr;
}

UD bool vclockwise(float2 a, float2 b) { float c = a.x * b.y - a.y * b.x; return c < 0; }

// getLineIntersection: vector2D.h:249-272 (float-float fast path, double
// pipeline when the fast path cannot decide; refmath.hpp)
UD bool line_intersection(float2 a, float2 b, float2 c, float2 d, float2* res)
{
	float x, y;
	const int r = line_intersection_ff(a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, &x, &y);
	if (r == 0) return false;
	if (r < 0 && !line_intersection_d(a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, &x, &y)) return false;
	*res = V(x, y);
	return true;
}

// ---------------------------------------------------------------------
// shared cost helpers (src/Engine/core/costFunction.cpp:173-227, 354-380)
// ---------------------------------------------------------------------
UD int solve_quadratic(float a, float b, float c, float* x1, float* x2)
{
	const float D = b * b - 4 * a * c;
	if (D < 0) return 0;
	if (D == 0) { *x1 = -b / 2 * a; return 1; }   // sic: costFunction.cpp:180
	const float m = -b / (2 * a);
	const float s = sqrtf(D) / (2 * a);
	*x1 = m + s;
	*x2 = m - s;
	return 2;
}

UD float ttc_pair(float2 p1, float2 v1, float r1, float2 p2, float2 v2, float r2)
{
	const float2 P = vsub(p1, p2);
	const float R = r1 + r2, RR = R * R;
	if (vsq(P) <= RR) return 0;
	const float2 Vd = vsub(v1, v2);
	const float a = vdot(Vd, Vd), b = 2 * vdot(P, Vd), c = vdot(P, P) - RR;
	float t1 = MAXF, t2 = MAXF;
	solve_quadratic(a, b, c, &t1, &t2);
	if (t1 < 0) t1 = MAXF;
	if (t2 < 0) t2 = MAXF;
	return fminr(t1, t2);
}

// nearestPointOnLine(pt, la, lb, onSegment = true): vector2D.h:274-296
UD float2 nearest_on_segment(float2 pt, float2 la, float2 lb)
{
	if (la.x == lb.x && la.y == lb.y) return la;
	const float2 line = vsub(la, lb);
	float k = vdot(vsub(pt, lb), line) / vsq(line);
	if (k > 1) k = 1;
	else if (k < 0) k = 0;
	return vadd(vmul(la, k), vmul(lb, 1 - k));
}
// distanceToLineSquared(pt, la, lb, true): vector2D.h:303-306
UD float dist2_to_segment(float2 pt, float2 la, float2 lb) { return vsq(vsub(pt, nearest_on_segment(pt, la, lb))); }

// ComputeTimeToCollision_LineSegmentInterior: costFunction.cpp:293-325
// (sinf: the host C library's, host_sinf).
UD float ttc_segment_interior(float2 p, float2 v, float r, float2 a, float2 b)
{
	if (dist2_to_segment(p, a, b) <= r * r) return 0;
	float2 X;
	if (!line_intersection(p, vadd(p, v), a, b, &X)) return MAXF;
	if (vdot(v, vsub(X, p)) < 0) return MAXF;
	// nearestPointOnLine(X, a, b, false, &onSegment): k in [0, 1]
	const float2 line = vsub(a, b);
	const float k = vdot(vsub(X, b), line) / vsq(line);
	if (!(k >= 0 && k <= 1)) return MAXF;
	const float speed = vmag(v);
	const float t = vmag(vsub(X, p)) / speed;
	const float ang = vangle_exact(v, vsub(b, a));
	const float sub = r / host_sinf(ang);
	const float tsub = sub / speed;
	return fmaxr(0.0f, t - tsub);
}

// ComputeTimeToCollision_LineSegment: costFunction.cpp:270-291
UD float ttc_segment(float2 p, float2 v, float r, float2 a, float2 b)
{
	const float t1 = ttc_pair(p, v, r, a, V(0, 0), 0);
	if (t1 == 0) return 0;
	if (a.x == b.x && a.y == b.y) return t1;
	const float t2 = ttc_pair(p, v, r, b, V(0, 0), 0);
	if (t2 == 0) return 0;
	const float ti = ttc_segment_interior(p, v, r, a, b);
	return fminr(fminr(t1, t2), ti);
}

// ttc_pair with P = p1 - p2 and c = |P|^2 - (r1 + r2)^2 given (the same
// values ttc_pair computes; |P|^2 <= RR exactly when c <= 0)
UD float ttc_pair_pre(float2 v1, float2 P, float c, float2 v2)
{
	if (c <= 0) return 0;
	const float2 Vd = vsub(v1, v2);
	const float a = vdot(Vd, Vd), b = 2 * vdot(P, Vd);
	float t1 = MAXF, t2 = MAXF;
	solve_quadratic(a, b, c, &t1, &t2);
	if (t1 < 0) t1 = MAXF;
	if (t2 < 0) t2 = MAXF;
	return fminr(t1, t2);
}

UD void ttca_dca(float2 p1, float2 v1, float r1, float2 p2, float2 v2, float r2, float* ttca_o, float* dca_o)
{
	const float2 dpc = vsub(p2, p1), dvc = vsub(v2, v1);
	const float dpMag = vmag(dpc);
	const float2 dp = vmul(vdiv(dpc, dpMag), dpMag - r1 - r2);
	const float2 nrm = V(-dpc.y, dpc.x);
	const float2 dv = vadd(dvc, vmul(nrm, vdot(nrm, dvc)));
	float ttca = (vsq(dv) == 0 ? 0 : -vdot(dp, dv) / vsq(dv));
	if (ttca < 0) ttca = 0;
	float dca = vmag(vadd(dp, vmul(dv, ttca)));
	if (dca < 0) dca = 0;
	*ttca_o = ttca;
	*dca_o = dca;
}

// RotateGradientToEuclideanCoordinates: costFunction.cpp:30-34
UD float2 rotate_gradient(float gth, float gs, float2 dir, float speed)
{
	float sn, cs;
	host_sincosf(gth, &sn, &cs);
	const float2 w = vadd(vmul(V(sn, 1 - cs), speed), V(0, gs));
	return V(dir.y * w.x + dir.x * w.y, -dir.x * w.x + dir.y * w.y);
}

#undef UD
}  // namespace umans
