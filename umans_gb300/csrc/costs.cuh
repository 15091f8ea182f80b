// Device cost functions: one restatement per reference CostFunction plugin.
//
// Each function evaluates the plugin's GetCost / force / gradient for one
// agent and one candidate velocity, reading the agent's sorted neighbour list
// (shared memory) and the neighbours' data (cell-sorted copies in global
// memory, L1/L2 resident).  The arithmetic follows the reference file:line
// cited at each function; devmath.cuh explains the FP64 handling.
#pragma once
#include "devmath.cuh"
#include "model.hpp"
#include "refmath.hpp"

namespace umans {

#define UD __device__ __forceinline__

// Neighbour access: ref = (displacement group << 28) | cell-sorted index.
struct NbView {
	const uint32_t* ref;     // [K]
	const float* d2;         // [K] PhantomAgent::distSqr
	int K;
	const float2* sP;        // cell-sorted positions
	const float2* sV;        // cell-sorted velocities
	const float4* sB;        // cell-sorted (pref.x, pref.y, radius, -)
	const float4* sE;        // cell-sorted (normalised pref.x, pref.y, speed, -)
	float W, H;              // toric world size (PhantomAgent offsets)
	// obstacle edges within range: (displacement group << 28) | edge index
	const float4* edges;
	const uint32_t* obs;
	int KO;
	// optional: the sample-invariant part of ttc_pair for every neighbour
	// within pp_range, in list order (P = p - p_j, |P|^2 - (r + r_j)^2,
	// v_j.x; v_j.y in pv), built once per agent before a sampling sweep
	const float4* pp = nullptr;
	const float* pv = nullptr;
	int KP = 0;
	float pp_range = -1.0f;
};

// PhantomAgent position offset of displacement group g (worldToric.cpp:61-79):
// 0 none, 1 (-W, -0), 2 (W, -0), 3 (-0, -H), 4 (-0, H).  Selected in
// registers (an indexed table would live in local memory).
UD float2 group_offset(uint32_t g, float W, float H)
{
	const float ox = g == 1 ? -W : (g == 2 ? W : (g == 0 ? 0.0f : -0.0f));
	const float oy = g == 3 ? -H : (g == 4 ? H : (g == 0 ? 0.0f : -0.0f));
	return V(ox, oy);
}

// displacement of group g (worldToric.cpp:65-76): 1 (W, 0), 2 (-W, 0),
// 3 (0, H), 4 (0, -H)
UD float2 group_disp(uint32_t g, float W, float H)
{
	const float dx = g == 1 ? W : (g == 2 ? -W : 0.0f);
	const float dy = g == 3 ? H : (g == 4 ? -H : 0.0f);
	return V(dx, dy);
}

// obstacle entry k: the edge, shifted by -displacement for displaced
// queries (worldToric.cpp:55-58)
UD void nb_seg(const NbView& N, int k, float2* a, float2* b)
{
	const uint32_t e = N.obs[k];
	const float4 E = N.edges[e & 0x0FFFFFFFu];
	*a = V(E.x, E.y);
	*b = V(E.z, E.w);
	const uint32_t g = e >> 28;
	if (g != 0) {
		const float2 d = group_disp(g, N.W, N.H);
		*a = vsub(*a, d);
		*b = vsub(*b, d);
	}
}

UD float2 nb_pos(const NbView& N, int k)
{
	const uint32_t r = N.ref[k];
	return vadd(N.sP[r & 0x0FFFFFFFu], group_offset(r >> 28, N.W, N.H));
}
UD float2 nb_vel(const NbView& N, int k) { return N.sV[N.ref[k] & 0x0FFFFFFFu]; }
UD float nb_radius(const NbView& N, int k) { return N.sB[N.ref[k] & 0x0FFFFFFFu].z; }
UD float4 nb_E(const NbView& N, int k) { return N.sE[N.ref[k] & 0x0FFFFFFFu]; }
UD float2 nb_pref(const NbView& N, int k)
{
	const float4 b = N.sB[N.ref[k] & 0x0FFFFFFFu];
	return V(b.x, b.y);
}

// The agent being updated (uniform across the warp).
struct AgentCtx {
	float2 pos, vel, pref, goal;
	float radius, prefspeed, maxspeed, maxacc, dt, relax;
	ExpExceptions ex;    // host-expf exceptions (refmath.hpp)
};

// ComputeTimeToFirstCollision: costFunction.cpp:229-268
UD float ttc_first(const AgentCtx& A, const NbView& N, float2 vel, float maxDist, bool ignoreCurrent)
{
	float minT = MAXF;
	const float md2 = maxDist * maxDist;
	if (N.pp != nullptr && maxDist == N.pp_range) {
		// the same pairs and the same values (ttc_pair_pre), from the cache
		for (int k = 0; k < N.KP; ++k) {
			const float4 q = N.pp[k];
			const float t = ttc_pair_pre(vel, V(q.x, q.y), q.z, V(q.w, N.pv[k]));
			if (ignoreCurrent && t == 0) continue;
			if (t < minT) minT = t;
		}
	} else {
		for (int k = 0; k < N.K; ++k) {
			if (N.d2[k] > md2) continue;
			const float t = ttc_pair(A.pos, vel, A.radius, nb_pos(N, k), nb_vel(N, k), nb_radius(N, k));
			if (ignoreCurrent && t == 0) continue;
			if (t < minT) minT = t;
		}
	}
	for (int k = 0; k < N.KO; ++k) {
		float2 a, b;
		nb_seg(N, k, &a, &b);
		if (dist2_to_segment(A.pos, a, b) > md2) continue;
		const float t = ttc_segment(A.pos, vel, A.radius, a, b);
		if (ignoreCurrent && t == 0) continue;
		if (t < minT) minT = t;
	}
	return minT;
}

// Pair-invariant terms of SocialForcesAvoidance for one agent and cost:
// -V0/sigma is the first factor of d_V as written (so precomputing it changes
// no rounding), |vel| is the agent's factor of the view test's lengths.
struct SfConst {
	float dtp, sigma, nV0s, vmag_vel;
};
UD SfConst sf_const(const AgentCtx& A, const CostDesc& c)
{
	SfConst K;
	K.dtp = c.p[0];
	K.sigma = c.p[2];
	K.nV0s = -c.p[1] / c.p[2];
	K.vmag_vel = vmag(A.vel);
	return K;
}

// angle(a, b) < thr (devmath.cuh angle_less) with |a| and |b| given
UD bool angle_less_m(float2 a, float2 b, float ma, float mb, float thr, float cos_thr)
{
	const float lf = ma * mb;
	if (lf == 0) return true;
	const float d = vdot(a, b);
	const float c = d / lf;
	if (c > cos_thr + 1e-6f) return true;
	if (c < cos_thr - 1e-6f && c > -0.9999f) return false;
	if (c <= -0.9999f) return -d > lf;
	return vangle_exact(a, b) < thr;
}

// SocialForcesAvoidance::ComputeAgentInteractionForce: SocialForcesAvoidance.cpp:26-110
// E = (Eb.x, Eb.y, vb): the neighbour's normalised preferred velocity and
// its speed (SocialForcesAvoidance.cpp:58-59), precomputed once per agent
UD float2 sf_force(const AgentCtx& A, const SfConst& K, float2 np, float4 E, float nr)
{
	const float2 R = vsub(A.pos, np);
	const float magR = vmag(R);
	if (magR <= A.radius + nr) return V(0, 0);
	const float vb = E.z;
	const float2 Eb = V(E.x, E.y);
	const float2 Vv = vmul(Eb, vb * K.dtp);
	const float magV = vmag(Vv);
	const float2 R2 = vsub(R, Vv);
	const float magR2 = vmag(R2);
	const float bSquared2 = sq_diff_d(magR + magR2, vb * K.dtp);
	if (bSquared2 <= 0) return V(0, 0);
	const float b = 0.5f * sqrtf(bSquared2);
	if (b < 0.001f) return V(0, 0);
	// cosAngle(R, Vv): the lengths are magR and magV
	const float lRV = magR * magV;
	const float cosRV = lRV == 0 ? 0.0f : vdot(R, Vv) / lRV;
	const float d_magR2 = 1 / (2 * magR2) * (2 * magR - 2 * magV * cosRV);
	const float d_bSquared2 = 2 * (magR + magR2) * (1 + d_magR2);
	const float d_b = (1 / (8 * b)) * d_bSquared2;
	const float d_V = K.nV0s * ref_expf(A.ex, -b / K.sigma) * d_b;
	const float2 F = vmul(vneg(R), d_V);
	// viewingAngleHalf = (float)(100 deg in rad); cos of it to 1e-8; |-R| = magR
	const float viewHalf = (float)(100.0 * REF_PI / 180.0);
	const float scale = angle_less_m(A.vel, vneg(R), K.vmag_vel, magR, viewHalf, -0.17364818f) ? 1.0f : 0.5f;
	return vmul(F, scale);
}

// SocialForcesAvoidance::ComputeObstacleInteractionForce:
// SocialForcesAvoidance.cpp:112-140 (U0 = p[3], R = p[4])
UD float2 sf_obstacle_force(const AgentCtx& A, const CostDesc& c, float2 a, float2 b)
{
	const float2 diff = vsub(A.pos, nearest_on_segment(A.pos, a, b));
	const float dist = vmag(diff);
	if (dist < 0.001f) return V(0, 0);
	const float U0 = c.p[3], R = c.p[4];
	const float d_U = -U0 / R * ref_expf(A.ex, -dist / R);
	return vmul(vneg(diff), d_U);
}

// PowerLaw::ComputeAgentInteractionForce: PowerLaw.cpp:28-66
UD float2 pl_force(const AgentCtx& A, const CostDesc& c, float2 np, float2 nv, float nr)
{
	const float k = c.p[0], tau0 = c.p[1];
	const float R = nr + A.radius;
	const float2 x = vsub(A.pos, np);
	const float2 v = vsub(A.vel, nv);
	const float a = vdot(v, v), b = -vdot(x, v), cc = vdot(x, x) - R * R;
	if (cc <= 0) return V(0, 0);
	const float d = b * b - a * cc;
	if (d <= 0) return V(0, 0);
	const float sqrtD = sqrtf(d);
	const float tau = (b - sqrtD) / a;
	if (tau < 0.001f) return V(0, 0);
	if (tau > tau0) return V(0, 0);
	const float comp1 = -k * ref_expf(A.ex, -tau / tau0) * (2 / tau + 1 / tau0) / (a * tau * tau);
	const float2 comp2 = vsub(v, vdiv(vadd(vmul(x, a), vmul(v, b)), sqrtD));
	return vmul(comp2, comp1);
}

// ---------------------------------------------------------------------
// per-candidate costs (sampling)
// ---------------------------------------------------------------------

// Karamouzas::getMaxDeviationAngle: Karamouzas.cpp:115-123 (tc_max stays 8,
// Karamouzas.h:58)
UD float karamouzas_maxdev(float ttc)
{
	const float tc_min = 2.5f, tc_mid = 6, tc_max = 8;
	const float d_min = 0.05f, d_mid = (float)(REF_PI / 6.0f), d_max = (float)(REF_PI / 2.0f);
	if (ttc <= 0 || ttc >= tc_max) return d_min;
	if (ttc < tc_min) {
		const double q = (double)((tc_min - ttc) / tc_min);
		return (float)__dadd_rn((double)d_mid, __dmul_rn(__dmul_rn(q, q), (double)(d_max - d_mid)));
	}
	if (ttc < tc_mid) return d_mid;
	return d_min + d_mid - (tc_max - ttc) / (tc_max - tc_mid);
}

// Karamouzas::GetCost: Karamouzas.cpp:28-113.  ttcp = TTC at the preferred
// velocity (sample invariant), maxdev/cosdev from it.  Split in three: the
// sample window (deviation angle, speed range; MAXF outside), the TTC sweep,
// and the cost terms.
UD bool karamouzas_window(const AgentCtx& A, float ttcp, float maxdev, float cosdev, float2 v, float speed)
{
	const float tc_min = 2.5f, tc_max = 8;
	if (angle_greater(v, A.pref, maxdev, cosdev)) return false;
	const float dS = fabsf(A.maxspeed - A.prefspeed), eps = 0.05f;
	float minS, maxS;
	if (ttcp <= 0 || ttcp >= tc_max) { minS = A.prefspeed - eps; maxS = A.prefspeed + eps; }
	else if (ttcp > 0 && ttcp < tc_min) { minS = 0; maxS = A.maxspeed + eps; }
	else { minS = A.prefspeed - dS - eps; maxS = A.prefspeed + dS + eps; }
	return !(speed < minS || speed > maxS);
}
UD float karamouzas_terms(const AgentCtx& A, const CostDesc& c, float2 v, float speed, float TTC)
{
	const float alpha = c.p[0], beta = c.p[1], gamma = c.p[2], delta = c.p[3], t_max = c.p[4];
	const float a = alpha * (1 - vcosangle(v, A.pref) / 2.0f);
	const float b = beta * fabsf(speed - vmag(A.vel)) / A.maxspeed;
	const float cc = gamma * vmag(vsub(v, A.pref)) / (2 * A.maxspeed);
	const float d = delta * fmaxr(0.0f, t_max - TTC) / t_max;
	return a + b + cc + d;
}
UD float cost_karamouzas(const AgentCtx& A, const NbView& N, const CostDesc& c, float ttcp, float maxdev,
                         float cosdev, float2 v)
{
	const float speed = vmag(v);
	if (!karamouzas_window(A, ttcp, maxdev, cosdev, v, speed)) return MAXF;
	return karamouzas_terms(A, c, v, speed, ttc_first(A, N, v, c.range, true));
}

// Moussaid::GetCost: Moussaid.cpp:28-62
UD float cost_moussaid(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	const float d_max = c.p[0];
	const float speed = vmag(v), prefSpeed = A.prefspeed;
	const float2 dir = vnorm(v);
	const float ttc = ttc_first(A, N, vmul(dir, prefSpeed), c.range, false);
	float DC = (ttc == MAXF ? MAXF : ttc * prefSpeed);
	if (DC > d_max) DC = d_max;
	float K = d_max * d_max + DC * DC - 2 * d_max * DC * vcosangle(dir, A.pref);
	K += 1;
	const float S = fminr(prefSpeed, DC / A.relax);
	const double q = (double)((S - speed) / S);
	return (float)__dmul_rn((double)K, __dadd_rn(1.0, __dmul_rn(q, q)));
}

// VanToll::GetCost: VanToll.cpp:29-64
UD float cost_vantoll(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	const float maxd = c.p[0];
	const float prefSpeed = vmag(A.pref), speed = vmag(v);
	const float cTTC = ttc_first(A, N, v, c.range, false);
	float dC = (cTTC == MAXF ? MAXF : cTTC * speed);
	if (dC > maxd) dC = maxd;
	const float a1 = vangle_exact(v, A.pref);
	const float a2 = fabsf(speed - prefSpeed) / prefSpeed;
	const float a3 = vangle_exact(v, A.vel);
	return 1 * (maxd - dC) + 1 * a1 + 1 * a2 + 1 * a3;
}

// PLEdestrians::GetCost: PLEdestrians.cpp:28-36
UD float cost_pledestrians(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	const float w_a = c.p[0], w_b = c.p[1], t_min = c.p[2], t_max = c.p[3];
	const float ttc = ttc_first(A, N, v, c.range, true);
	if (ttc < t_min) return MAXF;
	return t_max * (w_a + w_b * vsq(v)) + 2 * vmag(vsub(vsub(A.goal, A.pos), vmul(v, t_max))) * sqrtf(w_a * w_b);
}

// RVO::GetCost: RVO.cpp:28-44
UD float cost_rvo(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	if (vmag(v) > A.maxspeed) return MAXF;
	const float2 rv = vsub(vmul(v, 2), A.vel);
	const float2 vd = vsub(A.pref, v);
	const float minT = ttc_first(A, N, rv, c.range, true);
	return c.p[0] / minT + vmag(vd);
}

// ORCA::GetCost: ORCA.cpp:49-86 (lines: float4 point.xy, direction.xy)
UD float cost_orca(const AgentCtx& A, const float4* lines, int nlines, float2 v)
{
	float maxD = -MAXF;
	for (int k = 0; k < nlines; ++k) {
		const float4 L = lines[k];
		const float2 pm = vsub(V(L.x, L.y), v);
		maxD = fmaxr(maxD, L.z * pm.y - L.w * pm.x);
	}
	if (maxD <= 0) return vmag(vsub(v, A.pref));
	return maxD + 2 * A.maxspeed;
}

// Paris::GetCost: Paris.cpp:28-221
UD float cost_paris(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	const float w_a = c.p[0], w_b = c.p[1], t_max = c.p[2];
	const float2 dir = vnorm(v);
	const float rs = c.range * c.range;
	const float prefSpeed = vmag(A.pref);
	const float speed = vmag(v);
	float sumCP = 0, sumDev = 0;
	int cnt = 0;
	for (int k = 0; k < N.K; ++k) {
		if (N.d2[k] > rs) continue;
		const float2 np = nb_pos(N, k), nv = nb_vel(N, k);
		const float r1 = A.radius, r2 = nb_radius(N, k);
		float t1, s1, s2;
		float2 X;
		if (!line_intersection(A.pos, vadd(A.pos, dir), np, vadd(np, nv), &X)) {
			const float ttc = ttc_pair(A.pos, dir, r1, np, nv, r2);
			if (ttc > t_max) { t1 = t_max; s1 = 0; s2 = FLT_MAX; }
			else { t1 = 0; s1 = FLT_MAX; s2 = 0; }
		} else {
			float ta = ttc_pair(A.pos, A.vel, r1 + r2, X, V(0, 0), 0);
			if (ta > t_max) ta = t_max;
			if (ta == t_max) { t1 = t_max; s1 = 0; s2 = FLT_MAX; }
			else {
				float u1 = ttc_pair(np, nv, r1 + r2, X, V(0, 0), 0);
				if (u1 > t_max) u1 = t_max;
				float u2 = u1 + (r1 + r2) / vmag(nv);
				if (u2 > t_max) u2 = 0;
				const float distToX = vmag(vsub(X, A.pos));
				t1 = u1;
				s1 = distToX / u1;
				s2 = distToX / u2;
			}
		}
		const float cs = fminr(fmaxr(0.0f, 1.0f - s1 / prefSpeed), fmaxr(0.0f, (s2 - prefSpeed) / prefSpeed));
		const float cp = 1 - t1 / (t_max + w_b);
		sumCP += cs * cp;
		sumDev += fmaxr(0.0f, fmaxr((s1 - speed) / prefSpeed, (speed - s2) / prefSpeed));
		cnt++;
	}
	if (cnt > 0) sumCP /= (float)cnt;
	const float cangle = (float)(__dsub_rn(1.0, (double)vcosangle(dir, A.pref)) / 2.0);
	const float dirCost = w_a * sumCP + (1 - w_a) * cangle;
	const float diffToPref = vmag(vsub(v, A.pref));
	return 1000 * dirCost + sumDev + 0.001f * diffToPref;
}

// costForTtcaDca: TtcaDca.cpp:40-43
UD float ttcadca_pair_cost(float ttca, float dca, float sT, float sD)
{
	return exp_gauss(ttca / sT, dca / sD);
}

// TtcaDca::GetCost: TtcaDca.cpp:62-129
UD float cost_ttcadca(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	const float sA = c.p[0], sS = c.p[1], sT = c.p[2], sD = c.p[3];
	const float viewHalf = (float)(REF_PI / 2.0);
	const float rs = c.range * c.range;
	const float alpha = vangle_exact(v, A.pref);
	const float ds = vmag(v) - A.prefspeed;
	const float Ca = exp_gauss(alpha / sA, 0.0f);
	const float Cs = exp_gauss(ds / sS, 0.0f);
	const float move = 1 - (Ca + Cs) / 2.0f;
	float oc = 0, sc = 0;
	for (int k = 0; k < N.K; ++k) {
		if (N.d2[k] >= rs) continue;
		const float2 np = nb_pos(N, k);
		const float2 relPos = vsub(np, A.pos);
		if (angle_greater(relPos, A.vel, viewHalf, -4.3711388e-08f)) continue;
		float ttca, dca;
		const float nr = nb_radius(N, k);
		ttca_dca(A.pos, v, A.radius, np, nb_vel(N, k), nr, &ttca, &dca);
		const float dist = vmag(relPos) - A.radius - nr;
		const float scale = 1 / (dist * dist);
		sc += scale;
		oc += ttcadca_pair_cost(ttca, dca, sT, sD) * scale;
	}
	if (sc > 0) oc /= sc;
	return oc + move;
}

// FOEAvoidance Importance(): FOEAvoidance.cpp:41-49
UD float foe_importance(float ttc)
{
	if (ttc < 0.f || ttc > 10.f) return 0.f;
	const float t0 = 5, I0 = 10, a = -I0 / t0;
	const float I = a * ttc + I0;
	if (I < 0.1f) return 0.1f;
	if (I > 10.f) return 10.f;
	return I;
}

// FOEAvoidance::GetCost: FOEAvoidance.cpp:50-92
UD float cost_foe(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	if (viszero(v)) return 0;
	const float2 Vn = vnorm(v);
	const float rs = c.range * c.range;
	const double LN10 = 2.302585092994045684;   // log(10) in double
	float cost = 0;
	for (int k = 0; k < N.K; ++k) {
		if (N.d2[k] > rs) continue;
		const float2 dv = vsub(nb_vel(N, k), v), dp = vsub(nb_pos(N, k), A.pos);
		const float2 Vel = V(Vn.y * dv.x + -Vn.x * dv.y, Vn.x * dv.x + Vn.y * dv.y);
		const float2 Pos = V(Vn.y * dp.x + -Vn.x * dp.y, Vn.x * dp.x + Vn.y * dp.y);
		// (double)y < 0.1 <=> y < 0.1f;  (double)y > -0.01 <=> y >= -0.01f
		if (Pos.y < 0.1f || Vel.y >= -0.01f) continue;
		const float xf = Vel.x / Vel.y, xg = Pos.x / Pos.y, dx = xg - xf;
		const float ttc = -Pos.y / Vel.y;
		const float sigma = (float)__ddiv_rn((double)((A.radius + nb_radius(N, k)) / Pos.y), LN10);
		cost += foe_importance(ttc) * ref_expf(A.ex, -fabsf(dx) / sigma);
	}
	return cost;
}

#undef UD
}  // namespace umans
