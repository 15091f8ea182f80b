// Reverse-mode derivatives of the smooth force models, for the
// differentiable step.
//
// Each *_adj function recomputes the forward pair force exactly as costs.cuh
// does and then propagates the adjoint of that force (lf) back to its inputs:
// the relative position, the neighbour's velocity and goal direction, and the
// model parameters.  Branches (collision cut-offs, the view-angle factor, the
// time-to-collision window) are differentiated on the branch the forward pass
// took; neighbour lists are those of the forward pass.  The arithmetic is
// ordinary float: gradients are checked against FP64 finite differences, not
// bit for bit.
#pragma once
#include "costs.cuh"

namespace umans {

#define UDA __device__ __forceinline__

UDA float2 v2(float x, float y) { return make_float2(x, y); }
UDA float2 add2(float2 a, float2 b) { return v2(a.x + b.x, a.y + b.y); }
UDA float2 sub2(float2 a, float2 b) { return v2(a.x - b.x, a.y - b.y); }
UDA float2 mul2(float2 a, float s) { return v2(a.x * s, a.y * s); }
UDA float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }

// y = w / |w|: adjoint of w from the adjoint of y
UDA float2 normalize_adj(float2 w, float2 ly)
{
	const float m = sqrtf(dot2(w, w));
	if (!(m > 0)) return v2(0, 0);
	const float2 u = mul2(w, 1.0f / m);
	return mul2(sub2(ly, mul2(u, dot2(u, ly))), 1.0f / m);
}

// y = clampVector(x, L) (vector2D.h:241-247)
UDA float2 clamp_adj(float2 x, float L, float2 ly)
{
	const float m = sqrtf(dot2(x, x));
	if (m <= L) return ly;
	const float2 u = mul2(x, 1.0f / m);
	return mul2(sub2(ly, mul2(u, dot2(u, ly))), L / m);
}

struct SfAdj {
	float2 lR;      // adjoint of R = p_i - p_j
	float2 lvj;     // adjoint of the neighbour's velocity
	float2 lEb;     // adjoint of the neighbour's goal direction
	float lV0, lsigma;
};

// SocialForcesAvoidance::ComputeAgentInteractionForce (SocialForcesAvoidance.cpp:26-110)
UDA SfAdj sf_pair_adj(const AgentCtx& A, const CostDesc& c, float2 np, float2 nvel, float2 Eb, float nr, float2 lf)
{
	SfAdj o;
	o.lR = v2(0, 0); o.lvj = v2(0, 0); o.lEb = v2(0, 0); o.lV0 = 0; o.lsigma = 0;
	const float dtp = c.p[0], V0 = c.p[1], sigma = c.p[2];
	const float2 R = sub2(A.pos, np);
	const float magR = sqrtf(dot2(R, R));
	if (magR <= A.radius + nr) return o;
	const float vb = sqrtf(dot2(nvel, nvel));
	const float2 Vv = mul2(Eb, vb * dtp);
	const float magV = sqrtf(dot2(Vv, Vv));
	const float2 R2 = sub2(R, Vv);
	const float magR2 = sqrtf(dot2(R2, R2));
	const float S = magR + magR2, T = vb * dtp;
	// where S^2 - T^2 cancels, as the forward step: pow(S, 2) - pow(T, 2) in
	// double, rounded once (SocialForcesAvoidance.cpp:86); a plain float
	// difference would give a different b there, and the terms below go as 1/b
	float bSq = S * S - T * T;
	if (bSq < 0.05f * (S * S)) bSq = sq_diff_d(S, T);
	if (bSq <= 0) return o;
	const float b = 0.5f * sqrtf(bSq);
	if (b < 0.001f) return o;
	const float lens = magR * magV;
	const float cth = lens > 0 ? dot2(R, Vv) / lens : 0.0f;
	const float dmagR2 = (magR - magV * cth) / magR2;
	const float dbSq = 2 * S * (1 + dmagR2);
	const float db = dbSq / (8 * b);
	const float E = expf(-b / sigma);
	const float dV = -V0 / sigma * E * db;
	const float viewHalf = (float)(100.0 * REF_PI / 180.0);
	const float scale = angle_less(A.vel, v2(-R.x, -R.y), viewHalf, -0.17364818f) ? 1.0f : 0.5f;
	// f = scale * (-R) * dV
	float2 lR = mul2(lf, -scale * dV);
	const float ldV = -scale * dot2(R, lf);
	// dV = -(V0/sigma) E db
	o.lV0 = -(E * db / sigma) * ldV;
	float lsig = (V0 / (sigma * sigma)) * E * db * ldV;
	const float lE = -(V0 / sigma) * db * ldV;
	const float ldb = -(V0 / sigma) * E * ldV;
	// E = exp(-b / sigma)
	float lb = -(E / sigma) * lE;
	lsig += (E * b / (sigma * sigma)) * lE;
	o.lsigma = lsig;
	// db = dbSq / (8 b)
	const float ldbSq = ldb / (8 * b);
	lb += -dbSq / (8 * b * b) * ldb;
	// dbSq = 2 S (1 + dmagR2)
	float lS = 2 * (1 + dmagR2) * ldbSq;
	const float ldm = 2 * S * ldbSq;
	// dmagR2 = (magR - magV cth) / magR2
	float lmagR = ldm / magR2;
	float lmagV = -cth * ldm / magR2;
	const float lcth = -magV * ldm / magR2;
	float lmagR2 = -dmagR2 / magR2 * ldm;
	// cth = R.Vv / (magR magV)
	float2 lVv = v2(0, 0);
	if (lens > 0) {
		lR = add2(lR, mul2(sub2(mul2(Vv, 1.0f / lens), mul2(R, cth / (magR * magR))), lcth));
		lVv = add2(lVv, mul2(sub2(mul2(R, 1.0f / lens), mul2(Vv, cth / (magV * magV))), lcth));
	}
	// b = 0.5 sqrt(bSq); bSq = S^2 - T^2
	const float lbSq = lb / (8 * b);
	lS += 2 * S * lbSq;
	const float lT = -2 * T * lbSq;
	// S = magR + magR2
	lmagR += lS;
	lmagR2 += lS;
	// magR2 = |R - Vv|
	const float2 lR2 = mul2(R2, lmagR2 / magR2);
	lR = add2(lR, lR2);
	lVv = sub2(lVv, lR2);
	// magV = |Vv|
	if (magV > 0) lVv = add2(lVv, mul2(Vv, lmagV / magV));
	// Vv = Eb (vb dtp); T = vb dtp
	o.lEb = mul2(lVv, vb * dtp);
	const float lvb = dtp * dot2(Eb, lVv) + dtp * lT;
	// magR = |R|
	lR = add2(lR, mul2(R, lmagR / magR));
	o.lR = lR;
	if (vb > 0) o.lvj = mul2(nvel, lvb / vb);
	return o;
}

struct PlAdj {
	float2 lx;      // adjoint of x = p_i - p_j
	float2 lv;      // adjoint of v = v_i - v_j
	float lk, ltau0;
};

// float-float arithmetic for the PowerLaw adjoint (products exact by FMA)
UDA FF ffa_add(FF p, FF q)
{
	FF s = ff_two_sum(p.h, q.h);
	s.l += p.l + q.l;
	return ff_fast_two_sum(s.h, s.l);
}
UDA FF ffa_mul(FF p, FF q)
{
	FF r = ff_two_prod(p.h, q.h);
	r.l += p.h * q.l + p.l * q.h;
	return ff_fast_two_sum(r.h, r.l);
}
UDA float ffa_f(FF p) { return p.h + p.l; }

// a = v.v, b = -x.v, cc = x.x - R^2, d = b^2 - a cc, x, v and
// w = x + (cc / (b + sqrt(d))) v of a PowerLaw pair in float-float from the
// exact differences of the states (taken only for ill-conditioned pairs, off
// the common path: its registers stay out of the adjoint kernel)
struct PlExact { float a, b, cc, d; float2 x, v, w; };
__device__ __noinline__ PlExact pl_exact(float2 pi, float2 pj, float2 vi, float2 vj, float ri, float rj)
{
	const FF xx = ff_two_sum(pi.x, -pj.x), xy = ff_two_sum(pi.y, -pj.y);
	const FF vx = ff_two_sum(vi.x, -vj.x), vy = ff_two_sum(vi.y, -vj.y);
	const FF Rf = ff_two_sum(rj, ri);
	const FF aa = ffa_add(ffa_mul(vx, vx), ffa_mul(vy, vy));
	const FF bb = ffa_add(ffa_mul(xx, vx), ffa_mul(xy, vy));   // -b
	const FF cf = ffa_add(ffa_add(ffa_mul(xx, xx), ffa_mul(xy, xy)), ffa_mul(Rf, FF{ -Rf.h, -Rf.l }));
	const FF df = ffa_add(ffa_mul(bb, bb), ffa_mul(aa, FF{ -cf.h, -cf.l }));
	PlExact e;
	e.a = ffa_f(aa); e.b = -ffa_f(bb); e.cc = ffa_f(cf); e.d = ffa_f(df);
	e.x = v2(ffa_f(xx), ffa_f(xy));
	e.v = v2(ffa_f(vx), ffa_f(vy));
	const FF tf = FF{ e.d > 0 && e.b > 0 ? e.cc / (e.b + sqrtf(e.d)) : 0.0f, 0.0f };
	e.w = v2(ffa_f(ffa_add(xx, ffa_mul(tf, vx))), ffa_f(ffa_add(xy, ffa_mul(tf, vy))));
	return e;
}

// PowerLaw::ComputeAgentInteractionForce (PowerLaw.cpp:28-66).  The branches
// are decided on the forward step's own values (tau = (b - sqrt(d)) / a as
// the reference computes it); the derivative is taken of the same force in
// a form without cancellation: with u = b + sqrt(d), b - sqrt(d) = a cc / u,
// so tau = cc / u and comp2 = v - (a x + b v) / sqrt(d) = -a (x + tau v) /
// sqrt(d), and the force is
//   f = comp1 comp2 = k E h (x + tau v) / (tau^2 sqrt(d)),
//   E = exp(-tau / tau0), h = 2 / tau + 1 / tau0.
// (The written form subtracts nearly equal terms when the relative speed is
// small, which a float adjoint of it would amplify.)  Where d = b^2 - a cc,
// cc = x.x - R^2 or b = -x.v cancel, these are evaluated in float-float
// from the state (pl_exact): near a grazing collision (d << b^2; 4e-5 b^2
// was seen at the calibration density) the float discriminant keeps only a
// few bits, and the force goes as 1 / sqrt(d).
UDA PlAdj pl_pair_adj(const AgentCtx& A, const CostDesc& c, float2 np, float2 nvel, float nr, float2 lf)
{
	PlAdj o;
	o.lx = v2(0, 0); o.lv = v2(0, 0); o.lk = 0; o.ltau0 = 0;
	const float k = c.p[0], tau0 = c.p[1];
	const float R = nr + A.radius;
	const float2 x = sub2(A.pos, np);
	const float2 v = sub2(A.vel, nvel);
	const float a = dot2(v, v), b = -dot2(x, v), cc = dot2(x, x) - R * R;
	if (cc <= 0) return o;
	const float d = b * b - a * cc;
	if (d <= 0) return o;
	const float tau_f = (b - sqrtf(d)) / a;   // the forward step's value: its branches
	if (tau_f < 0.001f || tau_f > tau0) return o;
	// the same quantities, from the exact differences where they cancel
	float ae = a, be = b, ce = cc, de = d;
	float2 xe = x, ve = v;
	const float xx2 = dot2(x, x);
	const bool exact = d < 0.05f * b * b || cc < 0.05f * xx2 || b * b < 0.0025f * xx2 * a;
	float2 w;
	if (exact) {
		const PlExact e = pl_exact(A.pos, np, A.vel, nvel, A.radius, nr);
		ae = e.a; be = e.b; ce = e.cc; de = e.d; xe = e.x; ve = e.v; w = e.w;
		if (!(de > 0) || !(ae > 0) || !(be > 0)) return o;
	}
	const float sd = sqrtf(de);
	const float u = be + sd;
	const float tau = ce / u;
	const float E = expf(-tau / tau0);
	const float h = 2 / tau + 1 / tau0;
	// w = x + tau v (|w| = R at the collision)
	if (!exact) w = add2(x, mul2(v, tau));
	const float Gk = E * h / (tau * tau * sd);   // f = k Gk w
	const float G = k * Gk;
	// f = G w
	const float lG = dot2(w, lf);
	const float2 lw = mul2(lf, G);
	float2 lx = lw;
	float2 lv = mul2(lw, tau);
	float ltau = dot2(v, lw);
	// G = k E h / (tau^2 sd)
	o.lk = Gk * lG;
	const float lE = (k * h / (tau * tau * sd)) * lG;
	const float lh = (k * E / (tau * tau * sd)) * lG;
	ltau += -2 * (G / tau) * lG;
	float lsd = -(G / sd) * lG;
	// E = exp(-tau / tau0); h = 2 / tau + 1 / tau0
	ltau += -(E / tau0) * lE;
	float ltau0 = (E * tau / (tau0 * tau0)) * lE;
	ltau += -2 / (tau * tau) * lh;
	ltau0 += -1 / (tau0 * tau0) * lh;
	o.ltau0 = ltau0;
	// tau = cc / u, u = b + sd
	float lcc = ltau / u;
	const float lu = -(tau / u) * ltau;
	float lb = lu;
	lsd += lu;
	// sd = sqrt(d), d = b^2 - a cc
	const float ld = lsd / (2 * sd);
	lb += 2 * be * ld;
	const float la = -ce * ld;
	lcc += -ae * ld;
	// cc = x.x - R^2; b = -x.v; a = v.v
	lx = add2(lx, mul2(xe, 2 * lcc));
	lx = sub2(lx, mul2(ve, lb));
	lv = sub2(lv, mul2(xe, lb));
	lv = add2(lv, mul2(ve, 2 * la));
	o.lx = lx;
	o.lv = lv;
	return o;
}

// contact force term scale * (r_sum - |D|) * D / |D|, D = p_i - p_j
// (policy.cpp:107-141): adjoint of D
UDA float2 contact_adj(float2 D, float rsum, float scale, float2 lC)
{
	const float m = sqrtf(dot2(D, D));
	if (!(m > 0) || !(rsum - m > 0)) return v2(0, 0);
	const float2 n = mul2(D, 1.0f / m);
	return mul2(sub2(mul2(sub2(lC, mul2(n, dot2(n, lC))), rsum / m), lC), scale);
}

// Obstacle edge (a, b) seen from p: diff = p - nearest point of the segment
// (nearestPointOnLine with onSegment, vector2D.h:274-296) and whether the
// nearest point is interior (then d diff / d p = I - u u^T, u along the
// edge; at an end point or for a point-like edge it is I).
struct EdgeSeen { float2 diff, u; bool interior; };
UDA EdgeSeen edge_seen(float2 p, float2 a, float2 b)
{
	EdgeSeen r;
	r.interior = false;
	r.u = v2(0, 0);
	r.diff = vsub(p, nearest_on_segment(p, a, b));
	if (a.x == b.x && a.y == b.y) return r;
	const float2 line = vsub(a, b);
	const float k = vdot(vsub(p, b), line) / vsq(line);
	if (k > 0 && k < 1) {
		r.interior = true;
		r.u = mul2(line, 1.0f / sqrtf(dot2(line, line)));
	}
	return r;
}
// P^T v for P = d diff / d p
UDA float2 edge_proj(const EdgeSeen& e, float2 v)
{
	return e.interior ? sub2(v, mul2(e.u, dot2(e.u, v))) : v;
}

// SocialForcesAvoidance::ComputeObstacleInteractionForce
// (SocialForcesAvoidance.cpp:112-140): F = diff (U0/R) exp(-|diff|/R) for
// |diff| >= 0.001; adjoint of p from the adjoint lF of F
UDA float2 sf_obstacle_adj(const AgentCtx& A, const CostDesc& c, const EdgeSeen& e, float2 lF)
{
	const float dist = sqrtf(dot2(e.diff, e.diff));
	if (dist < 0.001f) return v2(0, 0);
	const float U0 = c.p[3], R = c.p[4];
	const float G = U0 / R * expf(-dist / R);
	// d F / d diff = G I + diff (dG/d dist) diff^T / dist, dG/d dist = -G/R
	const float2 ld = add2(mul2(lF, G), mul2(e.diff, -G / R * dot2(e.diff, lF) / dist));
	return edge_proj(e, ld);
}

// contact with an edge (policy.cpp:126-137): the agent-pair contact force
// with D = diff and r_j = 0
UDA float2 edge_contact_adj(const EdgeSeen& e, float radius, float scale, float2 lC)
{
	return edge_proj(e, contact_adj(e.diff, radius, scale, lC));
}

#undef UDA
}  // namespace umans
