// cost evaluation: warp helpers, analytic gradients, per-cost evaluation
// of velocity samples
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// ------------------------------------------------------------------------
// warp helpers
// ------------------------------------------------------------------------
// Adds f (this lane's term, used where `take` is set) to acc in lane order
// of the ballot, i.e. neighbour order.  All lanes end with the same acc.
__device__ __forceinline__ float2 ordered_accumulate(float2 acc, float2 f, bool take)
{
	unsigned m = __ballot_sync(0xffffffffu, take);
	while (m) {
		const int src = __ffs(m) - 1;
		const float fx = __shfl_sync(0xffffffffu, f.x, src);
		const float fy = __shfl_sync(0xffffffffu, f.y, src);
		acc.x += fx;
		acc.y += fy;
		m &= m - 1;
	}
	return acc;
}

// fx[0..K) summed by lane 0 and fy[0..K) by lane 1, in list order (the
// reference's sequential Vector2D sum), eight loads issued ahead of their
// additions; every lane returns both sums.
__device__ __forceinline__ float2 list_sum(const float* fx, const float* fy, int K, int lane)
{
	float acc = 0.0f;
	if (lane < 2) {
		const float* src = lane ? fy : fx;
		int k = 0;
		for (; k + 8 <= K; k += 8) {
			float v[8];
#pragma unroll
			for (int j = 0; j < 8; ++j) v[j] = src[k + j];
#pragma unroll
			for (int j = 0; j < 8; ++j) acc += v[j];
		}
		for (; k < K; ++k) acc += src[k];
	}
	return V(__shfl_sync(0xffffffffu, acc, 0), __shfl_sync(0xffffffffu, acc, 1));
}

__device__ float2 obstacle_force(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane);

// ObjectInteractionForces::ComputeForce: ObjectInteractionForces.cpp:26-48
// (agents only; obstacles add (0,0)); GoalReachingForce.cpp:26-29.
// Lanes evaluate one neighbour each into shared memory; lane 0 then adds the
// x terms and lane 1 the y terms in neighbour order, as the reference's
// sequential Vector2D sum does.
__device__ float2 compute_force(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane, float* fx, float* fy)
{
	if (c.kind == K_GOALREACHING) return vdiv(vsub(A.pref, A.vel), fmaxr(A.relax, A.dt));
	const float rs = c.range * c.range;
	if (c.kind == K_SOCIALFORCES) {
		const SfConst SK = sf_const(A, c);
		for (int k = lane; k < N.K; k += 32) {
			float2 f = V(0, 0);
			if (N.d2[k] <= rs) f = sf_force(A, SK, nb_pos(N, k), nb_E(N, k), nb_radius(N, k));
			fx[k] = f.x;
			fy[k] = f.y;
		}
	} else {
		for (int k = lane; k < N.K; k += 32) {
			float2 f = V(0, 0);
			if (N.d2[k] <= rs) f = pl_force(A, c, nb_pos(N, k), nb_vel(N, k), nb_radius(N, k));
			fx[k] = f.x;
			fy[k] = f.y;
		}
	}
	// neighbours beyond the cost's range hold +0.0 (see ordered_sums)
	__syncwarp();
	const float2 sum = list_sum(fx, fy, N.K, lane);
	__syncwarp();
	return vadd(sum, obstacle_force(A, N, c, lane));
}

// The obstacle edges within cost c's range, summed in list order
// (ObjectInteractionForces.cpp:40-45); PowerLaw has no obstacle force
// (PowerLaw.cpp:68-72: a zero vector each).
__device__ float2 obstacle_force(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane)
{
	const float rs = c.range * c.range;
	float2 obs = V(0, 0);
	if (c.kind == K_SOCIALFORCES) {
		for (int b0 = 0; b0 < N.KO; b0 += 32) {
			const int k = b0 + lane;
			bool take = false;
			float2 f = V(0, 0);
			if (k < N.KO) {
				float2 a, b;
				nb_seg(N, k, &a, &b);
				if (dist2_to_segment(A.pos, a, b) <= rs) { take = true; f = sf_obstacle_force(A, c, a, b); }
			}
			obs = ordered_accumulate(obs, f, take);
		}
	}
	return obs;
}

// ForceBasedFunction::ComputeTargetVelocity: ForceBasedFunction.cpp:48-52
__device__ __forceinline__ float2 target_velocity(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane,
                                                  float* fx, float* fy)
{
	return vadd(A.vel, vmul(vdiv(compute_force(A, N, c, lane, fx, fy), c.p[5]), A.dt));
}

__device__ __forceinline__ bool is_force_based(int kind)
{
	return kind == K_SOCIALFORCES || kind == K_POWERLAW || kind == K_GOALREACHING;
}

// Solver::createAgentOrcaLines + solveOrcaProgram: ORCASolver.cpp:61-171
__device__ float2 orca_solve(const AgentCtx& A, const NbView& N, const CostDesc& c, float4* lines, float4* proj,
                             int* nlines_out, int lane)
{
	const float tH = c.p[0];
	const float maxDistSq = c.range * c.range;
	int nl = 0;
	for (int base = 0; base < N.K; base += 32) {
		const int k = base + lane;
		const bool in = k < N.K && N.d2[k] <= maxDistSq;
		float4 out = make_float4(0, 0, 0, 0);
		if (in) {
			const float2 relPos = vsub(nb_pos(N, k), A.pos);
			const float2 relVel = vsub(A.vel, nb_vel(N, k));
			const float distSq = vsq(relPos);
			const float cR = A.radius + nb_radius(N, k);
			const float cRSq = cR * cR;
			float2 dir, u;
			if (distSq > cRSq) {
				const float2 w = vsub(relVel, vdiv(relPos, tH));
				const float wLenSq = vsq(w);
				const float dp1 = vdot(w, relPos);
				if (dp1 < 0.0f && dp1 * dp1 > cRSq * wLenSq) {
					const float wLen = sqrtf(wLenSq);
					const float2 unitW = vdiv(w, wLen);
					dir = V(unitW.y, -unitW.x);
					u = vmul(unitW, cR / tH - wLen);
				} else {
					const float leg = sqrtf(distSq - cRSq);
					if (det2(relPos, w) > 0.0f)
						dir = vdiv(V(relPos.x * leg - relPos.y * cR, relPos.x * cR + relPos.y * leg), distSq);
					else
						dir = vdiv(vmul(V(relPos.x * leg + relPos.y * cR, -relPos.x * cR + relPos.y * leg), -1), distSq);
					const float dp2 = vdot(relVel, dir);
					u = vsub(vmul(dir, dp2), relVel);
				}
			} else {
				const float2 w = vsub(relVel, vdiv(relPos, A.dt));
				const float wLen = vsq(w);   // sic: ORCASolver.cpp:161
				const float2 unitW = vdiv(w, wLen);
				dir = V(unitW.y, -unitW.x);
				u = vmul(unitW, cR / A.dt - wLen);
			}
			const float2 pt = vadd(A.vel, vmul(u, 0.5f));
			out = make_float4(pt.x, pt.y, dir.x, dir.y);
		}
		const unsigned m = __ballot_sync(0xffffffffu, in);
		if (in) lines[nl + __popc(m & ((1u << lane) - 1u))] = out;
		nl += __popc(m);
	}
	__syncwarp();
	float2 res;
	const int fail = lp2(lines, nl, A.maxspeed, A.pref, false, &res, lane);
	if (fail < nl) lp3(lines, nl, fail, A.maxspeed, &res, proj, lane);
	*nlines_out = nl;
	return res;
}

// ------------------------------------------------------------------------
// gradients (uniform across the warp)
// ------------------------------------------------------------------------
// TtcaDca::GetGradient: TtcaDca.cpp:131-262
// Sums of per-neighbour terms in neighbour order: lane j < nsum adds z_j[0..K)
// sequentially (entries of neighbours that contribute nothing hold +0.0,
// which leaves a sum that starts at +0.0 unchanged: x + (+0) = x for x != -0,
// and such sums never reach -0.0).  Returns the sums in s[0..nsum).
__device__ __forceinline__ void ordered_sums(const float* z0, const float* z1, const float* z2, int nsum, int K,
                                             int lane, float* s)
{
	__syncwarp();
	float acc = 0.0f;
	if (lane < nsum) {
		const float* src = lane == 0 ? z0 : (lane == 1 ? z1 : z2);
		for (int k = 0; k < K; ++k) acc += src[k];
	}
	s[0] = __shfl_sync(0xffffffffu, acc, 0);
	s[1] = __shfl_sync(0xffffffffu, acc, 1);
	s[2] = __shfl_sync(0xffffffffu, acc, 2);
	__syncwarp();
}

// TtcaDca::GetGradient (TtcaDca.cpp:130-223): the per-neighbour terms
// lane-parallel into z0..z2, then the reference's three sums in order
__device__ float2 grad_ttcadca(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v, int lane, float* z0,
                               float* z1, float* z2)
{
	const float sA = c.p[0], sS = c.p[1], sT = c.p[2], sD = c.p[3];
	const float viewHalf = (float)(REF_PI / 2.0);
	const float eps = 0.001f;
	const float rs = c.range * c.range;
	for (int k = lane; k < N.K; k += 32) {
		z0[k] = 0.0f; z1[k] = 0.0f; z2[k] = 0.0f;
		if (N.d2[k] > rs) continue;
		const float2 np = nb_pos(N, k);
		const float nr = nb_radius(N, k);
		const float2 dpc = vsub(np, A.pos), dvc = vsub(nb_vel(N, k), v);
		if (angle_greater(dpc, A.vel, viewHalf, -4.3711388e-08f)) continue;
		const float dpMag = vmag(dpc);
		const float2 dp = vmul(vdiv(dpc, dpMag), dpMag - A.radius - nr);
		const float2 nrm = V(-dpc.y, dpc.x);
		const float2 dv = vadd(dvc, vmul(nrm, vdot(nrm, dvc)));
		const float dvSq = vsq(dv);
		float ttca = (dvSq == 0 ? 0 : -vdot(dp, dv) / dvSq);
		if (ttca < 0) ttca = 0;
		const float2 vdca = vadd(dp, vmul(dv, ttca));
		float dca = vmag(vdca);
		if (dca < 0) dca = 0;
		if (dvSq <= eps) continue;
		const float2 VelRot = V(dv.y, -dv.x);
		const float VelMag = sqrtf(dvSq);
		const float2 VelNorm = vdiv(dv, VelMag);
		float gTA = 0, gTS = 0;
		if (fabsf(ttca) > eps) {
			const float2 rel = vadd(dp, vmul(dv, 2 * ttca));
			gTA = -vdot(rel, VelRot) / dvSq;
			gTS = vdot(rel, VelNorm) / dvSq;
		}
		float gDA = 0, gDS = 0;
		if (fabsf(dca) > eps) {
			gDA = vdot(vdca, vadd(vmul(dv, gTA), vmul(VelRot, ttca))) / dca;
			gDS = vdot(vdca, vsub(vmul(dv, gTS), vmul(VelNorm, ttca))) / dca;
		}
		const float cost = ttcadca_pair_cost(ttca, dca, sT, sD);
		const float tf = ttca / (sT * sT), df = dca / (sD * sD);
		const float gCS = -cost * (gTS * tf + gDS * df);
		const float gCA = -cost * (gTA * tf + gDA * df);
		const float scale = 1 / vsq(dp);
		z0[k] = gCA * scale;
		z1[k] = gCS * scale;
		z2[k] = scale;
	}
	float sums[3];
	ordered_sums(z0, z1, z2, 3, N.K, lane, sums);
	float GradTh = sums[0], GradS = sums[1];
	const float total = sums[2];
	if (total > 0) { GradTh /= total; GradS /= total; }
	// getMovementCostGradient: TtcaDca.cpp:54-60 (counterClockwiseAngle)
	float alpha = vangle_exact(v, A.pref);
	if (vclockwise(v, A.pref)) alpha = -alpha;
	const float ds = vmag(v) - A.prefspeed;
	const double qa = (double)(alpha / sA), qs = (double)(ds / sS);
	const double DCa = __dmul_rn((double)(alpha / (2 * sA * sA)), exp(-0.5 * __dmul_rn(qa, qa)));
	const double DCs = __dmul_rn((double)(ds / (2 * sS * sS)), exp(-0.5 * __dmul_rn(qs, qs)));
	GradTh += (float)DCa;
	GradS += (float)DCs;
	if ((double)vsq(v) < 0.01)
		return rotate_gradient(GradTh, GradS, vnorm(A.pref), vmag(A.pref));
	return rotate_gradient(GradTh, GradS, vnorm(v), vmag(v));
}

// FOEAvoidance::GetGradient: FOEAvoidance.cpp:94-143
__device__ float2 grad_foe(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v, int lane, float* z0,
                           float* z1)
{
	if (viszero(v)) return V(0, 0);
	const float2 Vn = vnorm(v);
	const float rs = c.range * c.range;
	const double LN10 = 2.302585092994045684;
	for (int k = lane; k < N.K; k += 32) {
		z0[k] = 0.0f; z1[k] = 0.0f;
		if (N.d2[k] > rs) continue;
		const float2 dv = vsub(nb_vel(N, k), v), dp = vsub(nb_pos(N, k), A.pos);
		const float2 Vel = V(Vn.y * dv.x + -Vn.x * dv.y, Vn.x * dv.x + Vn.y * dv.y);
		const float2 Pos = V(Vn.y * dp.x + -Vn.x * dp.y, Vn.x * dp.x + Vn.y * dp.y);
		if (Pos.y < 0.1f || Vel.y >= -0.01f) continue;
		const float xf = Vel.x / Vel.y, xg = Pos.x / Pos.y, dx = xg - xf;
		const float ttc = -Pos.y / Vel.y;
		const float sigma = (float)__ddiv_rn((double)((A.radius + nb_radius(N, k)) / Pos.y), LN10);
		const float sg = (float)((0 < dx) - (dx < 0));
		const float E = foe_importance(ttc) * ref_expf(A.ex, -fabsf(dx) / sigma);
		z0[k] = E * sg * (xf * xf - xg * xg - (vmag(v) / (-Vel.y))) / sigma;
		z1[k] = E * sg * (-xf / (-Vel.y)) / sigma;
	}
	float sums[3];
	ordered_sums(z0, z1, z1, 2, N.K, lane, sums);
	float gt = sums[0];
	const float gv = sums[1];
	if (gt < -0.1f) gt = -0.1f;
	else if (gt > 0.1f) gt = 0.1f;
	float sn, cs;
	host_sincosf(gt, &sn, &cs);
	const float2 w = vadd(vmul(V(sn, 1 - cs), vmag(v)), V(0, gv));
	return V(-Vn.y * w.x + -Vn.x * w.y, -(-Vn.x) * w.x + -Vn.y * w.y);
}

}  // namespace umans
// cost-function plugins: their device functions may use the gradient
// helpers above (grad_foe, ordered_sums, ...)
#include "plugins.cuh"
namespace umans {

// ------------------------------------------------------------------------
// per-cost evaluation (sampling / finite differences)
// ------------------------------------------------------------------------
struct CostPrep {
	float2 target[MAX_COSTS];    // force-based target velocity
	float ttcp[MAX_COSTS];       // Karamouzas TTC at the preferred velocity
	float maxdev[MAX_COSTS], cosdev[MAX_COSTS];
	const float4* lines;         // ORCA lines
	int nlines;
	float2 orca_v;
};

__device__ float eval_cost(const AgentCtx& A, const NbView& N, const CostDesc& c, const CostPrep& P, int ci, float2 v)
{
	switch (c.kind) {
	case K_SOCIALFORCES: case K_POWERLAW: case K_GOALREACHING:
		return 0.5f * vsq(vsub(v, P.target[ci])) / A.dt;   // ForceBasedFunction.cpp:26-30
	case K_KARAMOUZAS: return cost_karamouzas(A, N, c, P.ttcp[ci], P.maxdev[ci], P.cosdev[ci], v);
	case K_MOUSSAID: return cost_moussaid(A, N, c, v);
	case K_VANTOLL: return cost_vantoll(A, N, c, v);
	case K_PLEDESTRIANS: return cost_pledestrians(A, N, c, v);
	case K_RVO: return cost_rvo(A, N, c, v);
	case K_ORCA: return cost_orca(A, P.lines, P.nlines, v);
	case K_PARIS: return cost_paris(A, N, c, v);
	case K_TTCADCA: return cost_ttcadca(A, N, c, v);
	case K_FOE: return cost_foe(A, N, c, v);
	case K_GENERIC: return 0;   // GenericCost::GetCost: GenericCost.cpp:27-31
	}
	if (c.kind >= K_PLUGIN0) return plugin_cost(c.kind - K_PLUGIN0, A, N, c, v);
	return 0;
}

__device__ __forceinline__ uint32_t mulmod(uint32_t a, uint32_t b)
{
	return (uint32_t)(((uint64_t)a * b) % LCG_M);
}
// generate_canonical<float,24> on minstd_rand0 state x, then a + u*(b-a)
__device__ __forceinline__ float rng_uniform(uint32_t x, float a, float b)
{
	const float sum = (float)(x - 1u);
	float ret = sum / 2147483648.0f;
	if (ret >= 1.0f) ret = 0.99999994f;   // nextafter(1, 0)
	return ret * (b - a) + a;
}

// CostFunction::ApproximateGlobalMinimumBySampling: costFunction.cpp:66-164.
// Samples are spread over lanes; the argmin keeps the first strict minimum.
// Samples of the Karamouzas window swept together (independent chains).
// Measured on a 100k-agent corridor (k_agent<3>, ms per step):
// 2: 17.9, 3: 17.3, 4: 16.8, 5: 17.1, 6: 17.2, 8: 20.5, 10: 23.5.
#ifndef UMANS_KS
#define UMANS_KS 4
#endif
constexpr int KS = UMANS_KS;

// KARA: every policy of the launch samples a regular schedule with one
// Karamouzas cost (the general sampler is compiled out)
template <bool KARA = false>
__device__ float2 sample_min(const DevState& S, const AgentCtx& A, const NbView& N, const PolicyDesc& pol,
                             const CostPrep& P, uint32_t rng0, int lane, float4* pair4, float* pairv)
{
	float2 base = V(0, 0);
	if (pol.table_base == 1) base = A.vel;
	float radius;
	if (pol.table_radius == 0) radius = A.prefspeed;
	else if (pol.table_radius == 1) radius = A.maxspeed;
	else radius = fminr(2.0f * A.maxspeed, A.maxacc * A.dt);
	float2 dir = V(1, 0);
	if (pol.table_dir == 1) dir = vnorm(A.vel);
	else if (pol.table_dir == 2) dir = vnorm(A.pref);
	const float dL = radius / (float)pol.len_divisor;
	const int ncost = pol.single_cost ? 1 : pol.ncost;
	float bestC = MAXF;
	int bestI = 0x7fffffff;
	if (KARA || (ncost == 1 && pol.cost[0].kind == K_KARAMOUZAS && !pol.table_random)) {
		// Karamouzas alone: most samples fall outside its window (cost MAXF);
		// the lanes test the windows of 32 samples at a time, then the warp
		// sweeps the neighbours for each sample inside, in sample order.
		const CostDesc& c = pol.cost[0];
		const float coeff = pol.single_cost ? 1.0f : c.coeff;
		const float outside = 0.0f + coeff * MAXF;   // the sum of one term, as below
		int first_out = 0x7fffffff;
		// the sample-invariant part of every pair within the cost's range,
		// compacted into this warp's scratch: ttc_pair's P = p - p_j and
		// c = |P|^2 - (r + r_j)^2 (c <= 0 exactly when |P|^2 <= (r + r_j)^2),
		// and the neighbour's velocity
		int KP = 0;
		{
			const float md2 = c.range * c.range;
			for (int b0 = 0; b0 < N.K; b0 += 32) {
				const int k = b0 + lane;
				const bool inr = k < N.K && !(N.d2[k] > md2);
				const unsigned m = __ballot_sync(0xffffffffu, inr);
				if (inr) {
					const float2 Pd = vsub(A.pos, nb_pos(N, k));
					const float R = A.radius + nb_radius(N, k);
					const float2 vj = nb_vel(N, k);
					const int idx = KP + __popc(m & ((1u << lane) - 1u));
					pair4[idx] = make_float4(Pd.x, Pd.y, vdot(Pd, Pd) - R * R, vj.x);
					pairv[idx] = vj.y;
				}
				KP += __popc(m);
			}
			__syncwarp();
		}
		unsigned long long n_in = 0;
		for (int i0 = 0; i0 < pol.nsamples; i0 += 32) {
			const int i = i0 + lane;
			float2 v = V(0, 0);
			float speed = 0;
			bool in = false, valid = i < pol.nsamples;
			if (valid) {
				const SampleEntry e = S.table[pol.table_offset + i];
				v = vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
				speed = vmag(v);
				in = karamouzas_window(A, P.ttcp[0], P.maxdev[0], P.cosdev[0], v, speed);
			}
			const unsigned out_mask = __ballot_sync(0xffffffffu, valid && !in);
			if (out_mask && first_out == 0x7fffffff) first_out = i0 + __ffs(out_mask) - 1;
			// KS samples inside the window at a time: their sweeps share the
			// pair loads and run as independent chains
			unsigned m = __ballot_sync(0xffffffffu, in);
			n_in += __popc(m);
			while (m) {
				int si[KS];
				float2 sv[KS];
				float ssp[KS], T[KS];
#pragma unroll
				for (int j = 0; j < KS; ++j) {
					si[j] = m ? __ffs(m) - 1 : -1;
					if (m) m &= m - 1;
					const int src = si[j] < 0 ? si[0] : si[j];
					sv[j] = V(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
					ssp[j] = __shfl_sync(0xffffffffu, speed, src);
					T[j] = MAXF;
				}
				// ComputeTimeToFirstCollision over the pairs (ignoring current
				// collisions): minima, split over the lanes
				for (int k = lane; k < KP; k += 32) {
					const float4 q = pair4[k];
					const float2 P2 = V(q.x, q.y), v2 = V(q.w, pairv[k]);
#pragma unroll
					for (int j = 0; j < KS; ++j) {
						const float t = ttc_pair_pre(sv[j], P2, q.z, v2);
						if (t != 0 && t < T[j]) T[j] = t;
					}
				}
				// obstacle edges within the cost's range
				for (int k = lane; k < N.KO; k += 32) {
					float2 a, b;
					nb_seg(N, k, &a, &b);
					if (dist2_to_segment(A.pos, a, b) > c.range * c.range) continue;
					for (int j = 0; j < KS; ++j) {
						const float t = ttc_segment(A.pos, sv[j], A.radius, a, b);
						if (t != 0 && t < T[j]) T[j] = t;
					}
				}
#pragma unroll
				for (int j = 0; j < KS; ++j)
					for (int o = 16; o > 0; o >>= 1) {
						const float x = __shfl_xor_sync(0xffffffffu, T[j], o);
						if (x < T[j]) T[j] = x;
					}
				// costs in sample order: the first strict minimum is kept
#pragma unroll
				for (int j = 0; j < KS; ++j) {
					if (si[j] < 0) break;
					const float tc = 0.0f + coeff * karamouzas_terms(A, c, sv[j], ssp[j], T[j]);
					if (tc < bestC) { bestC = tc; bestI = i0 + si[j]; }
				}
			}
		}
		if (S.counters && lane == 0) {
			atomicAdd(&S.counters[0], n_in);
			atomicAdd(&S.counters[1], n_in * (unsigned long long)KP);
			atomicAdd(&S.counters[2], 1ull);
		}
		// samples outside the window all cost `outside`; like every sample
		// they count only below the initial best (MAXF), and then the first
		// of them competes with the best inside on (cost, index)
		if (first_out != 0x7fffffff && outside < MAXF &&
		    (outside < bestC || (outside == bestC && first_out < bestI))) {
			bestC = outside;
			bestI = first_out;
		}
		if (bestI == 0x7fffffff) return V(0, 0);
		const SampleEntry e = S.table[pol.table_offset + bestI];
		return vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
	}
	// costs that take the time to first collision per sample: the
	// sample-invariant pair terms once per agent (not with ORCA, whose lines
	// use the same scratch)
	NbView NC = N;
	{
		float cr = -1.0f;
		bool orca = false;
		for (int ci = 0; ci < ncost; ++ci) {
			const int kd = pol.cost[ci].kind;
			orca |= kd == K_ORCA;
			if (cr < 0.0f && (kd == K_RVO || kd == K_VANTOLL || kd == K_PLEDESTRIANS || kd == K_MOUSSAID ||
			                  kd == K_KARAMOUZAS))
				cr = pol.cost[ci].range;
		}
		if (cr >= 0.0f && !orca) {
			const float md2 = cr * cr;
			int KP = 0;
			for (int b0 = 0; b0 < N.K; b0 += 32) {
				const int k = b0 + lane;
				const bool inr = k < N.K && !(N.d2[k] > md2);
				const unsigned m = __ballot_sync(0xffffffffu, inr);
				if (inr) {
					const float2 Pd = vsub(A.pos, nb_pos(N, k));
					const float R = A.radius + nb_radius(N, k);
					const float2 vj = nb_vel(N, k);
					const int idx = KP + __popc(m & ((1u << lane) - 1u));
					pair4[idx] = make_float4(Pd.x, Pd.y, vdot(Pd, Pd) - R * R, vj.x);
					pairv[idx] = vj.y;
				}
				KP += __popc(m);
			}
			__syncwarp();
			NC.pp = pair4;
			NC.pv = pairv;
			NC.KP = KP;
			NC.pp_range = cr;
		}
	}
	for (int i = lane; i < pol.nsamples; i += 32) {
		float2 v;
		const int d0 = i * pol.draws;   // draws before this sample
		if (pol.table_random) {
			const float ma = pol.max_angle;
			const uint32_t x1 = mulmod(S.lcgpow[d0 + 1], rng0);
			const uint32_t x2 = mulmod(S.lcgpow[d0 + 2], rng0);
			const float ra = rng_uniform(x1, -ma, ma);
			const float rl = rng_uniform(x2, 0, radius);
			float sn, cs;
			host_sincosf(ra, &sn, &cs);
			v = vadd(base, vmul(vrot_cs(dir, cs, sn), rl));
		} else {
			const SampleEntry e = S.table[pol.table_offset + i];
			v = vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
		}
		float tc = 0;
		int jr = d0 + (pol.table_random ? 2 : 0);
		for (int ci = 0; ci < ncost; ++ci) {
			const float coeff = pol.single_cost ? 1.0f : pol.cost[ci].coeff;
			float cv;
			if (pol.cost[ci].kind == K_RANDOM)   // RandomFunction::GetCost: RandomFunction.cpp:25-28
				cv = rng_uniform(mulmod(S.lcgpow[++jr], rng0), -1, 1);
			else
				cv = eval_cost(A, NC, pol.cost[ci], P, ci, v);
			tc += coeff * cv;
		}
		if (tc < bestC) { bestC = tc; bestI = i; }
	}
	for (int o = 16; o > 0; o >>= 1) {
		const float oc = __shfl_xor_sync(0xffffffffu, bestC, o);
		const int oi = __shfl_xor_sync(0xffffffffu, bestI, o);
		if (oc < bestC || (oc == bestC && oi < bestI)) { bestC = oc; bestI = oi; }
	}
	if (bestI == 0x7fffffff) return V(0, 0);
	// every lane rebuilds the winning candidate
	const int i = bestI;
	if (pol.table_random) {
		const float ma = pol.max_angle;
		const uint32_t x1 = mulmod(S.lcgpow[i * pol.draws + 1], rng0);
		const uint32_t x2 = mulmod(S.lcgpow[i * pol.draws + 2], rng0);
		const float ra = rng_uniform(x1, -ma, ma);
		const float rl = rng_uniform(x2, 0, radius);
		float sn, cs;
		host_sincosf(ra, &sn, &cs);
		return vadd(base, vmul(vrot_cs(dir, cs, sn), rl));
	}
	const SampleEntry e = S.table[pol.table_offset + i];
	return vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
}

}  // namespace umans
