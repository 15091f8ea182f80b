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
	const float bSq = S * S - T * T;
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

// PowerLaw::ComputeAgentInteractionForce (PowerLaw.cpp:28-66)
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
	const float sd = sqrtf(d);
	const float tau = (b - sd) / a;
	if (tau < 0.001f || tau > tau0) return o;
	const float E = expf(-tau / tau0);
	const float h = 2 / tau + 1 / tau0;
	const float comp1 = -k * E * h / (a * tau * tau);
	const float2 q = add2(mul2(x, a), mul2(v, b));
	const float2 comp2 = sub2(v, mul2(q, 1.0f / sd));
	// f = comp1 comp2
	const float lc1 = dot2(comp2, lf);
	const float2 lc2 = mul2(lf, comp1);
	// comp2 = v - q / sd
	float2 lv = lc2;
	const float2 lq = mul2(lc2, -1.0f / sd);
	float lsd = dot2(q, lc2) / (sd * sd);
	float la = dot2(x, lq);
	float2 lx = mul2(lq, a);
	float lb = dot2(v, lq);
	lv = add2(lv, mul2(lq, b));
	// comp1 = -k E h / (a tau^2)
	o.lk = (comp1 / k) * lc1;
	const float lE = (comp1 / E) * lc1;
	const float lh = (comp1 / h) * lc1;
	la += -(comp1 / a) * lc1;
	float ltau = -2 * (comp1 / tau) * lc1;
	// h = 2/tau + 1/tau0
	ltau += -2 / (tau * tau) * lh;
	float ltau0 = -1 / (tau0 * tau0) * lh;
	// E = exp(-tau / tau0)
	ltau += -(E / tau0) * lE;
	ltau0 += (E * tau / (tau0 * tau0)) * lE;
	o.ltau0 = ltau0;
	// tau = (b - sd) / a
	lb += ltau / a;
	lsd += -ltau / a;
	la += -(tau / a) * ltau;
	// sd = sqrt(d); d = b^2 - a cc
	const float ld = lsd / (2 * sd);
	lb += 2 * b * ld;
	la += -cc * ld;
	const float lcc = -a * ld;
	// cc = x.x - R^2; b = -x.v; a = v.v
	lx = add2(lx, mul2(x, 2 * lcc));
	lx = sub2(lx, mul2(v, lb));
	lv = sub2(lv, mul2(x, lb));
	lv = add2(lv, mul2(v, 2 * la));
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
