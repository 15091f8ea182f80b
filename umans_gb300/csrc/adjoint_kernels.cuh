// differentiable form: adjoint kernels, loss and its seed
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// ------------------------------------------------------------------------
// differentiable form
// ------------------------------------------------------------------------
// Per-agent terms that the neighbours' adjoints read, from the state at the
// start of the step being reversed: the normalised goal direction Eb (as the
// scatter computes it for SocialForcesAvoidance), 1/|goal - pos| (0 at the
// goal: Eb is then constant) and the speed.
__global__ void k_adj_prep(DevState S)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= S.n) return;
	const float2 d = vsub(S.goal[i], S.a_pos[i]);
	const float4 prm = S.prm[i];
	const float2 v = S.a_vel[i];
	float2 eb = V(0, 0);
	float invw = 0;
	if (!(vsq(d) <= prm.x * prm.x)) {
		eb = vnorm(vmul(vnorm(d), prm.y));
		if (!viszero(eb)) invw = 1.0f / vmag(d);
	}
	S.adj_nb[i] = make_float4(eb.x, eb.y, invw, vmag(v));
}

// Adjoint of one step for policies made of SocialForcesAvoidance, PowerLaw
// and GoalReachingForce under the gradient method, with the neighbour lists
// the forward step recorded.  One warp per agent (list order), one lane per
// neighbour: the pair's force adjoints (every cost) and contact adjoint are
// formed together, the agent's own terms summed over the warp, and the
// neighbour's terms added to its adjoint with one atomic per nonzero
// component.  The parameters' adjoints (V0, sigma, k, tau0) are summed per
// scenario.
// this lane's share of the obstacle terms of an agent's position adjoint:
// SocialForces obstacle forces (compute_force) and contact with edges, over
// the edge list regathered from the reversed step's start state (not
// inlined, to keep k_adjoint's registers for scenarios without obstacles)
__device__ __noinline__ float2 obstacle_adjoint(const DevState& S, const ScenDesc& sd, const PolicyDesc& pol,
                                                const AgentCtx& A, int gw, int lane, bool moving, bool contact,
                                                float2 la, float2 lC)
{
	NbView N;
	N.edges = S.edges; N.W = sd.width; N.H = sd.height;
	uint32_t* ol = S.obs_list + (size_t)gw * S.max_obs;
	N.obs = ol;
	N.KO = gather_obstacles(S, sd, A.pos, pol.range, lane, ol);
	float2 lp = v2(0, 0);
	for (int k = lane; k < N.KO; k += 32) {
		float2 a, b;
		nb_seg(N, k, &a, &b);
		const EdgeSeen es = edge_seen(A.pos, a, b);
		if (moving)
			for (int c = 0; c < pol.ncost; ++c) {
				const CostDesc& cd = pol.cost[c];
				if (cd.kind != K_SOCIALFORCES || dist2_to_segment(A.pos, a, b) > cd.range * cd.range) continue;
				lp = add2(lp, sf_obstacle_adj(A, cd, es, mul2(la, cd.coeff / cd.p[5])));
			}
		if (contact) lp = add2(lp, edge_contact_adj(es, A.radius, pol.contact_scale, lC));
	}
	__syncwarp();
	return lp;
}

template <bool OBST>
__global__ void __launch_bounds__(128, 5) k_adjoint(DevState S)   // 5 blocks per SM (the launch)
{
	const int lane = threadIdx.x & 31;
	const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int nw = (gridDim.x * blockDim.x) >> 5;
	for (int i = gw; i < S.n; i += nw) {
		const int sc = S.agent_scen[i];
		const ScenDesc sd = S.scen[sc];
		const PolicyDesc& pol = S.pols[S.pol[i]];
		const float4 prm = S.prm[i];
		AgentCtx A;
		A.pos = S.a_pos[i]; A.vel = S.a_vel[i]; A.goal = S.goal[i];
		A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
		A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;
		const float dt = sd.dt;
		const float2 lp = S.lam_out_p[i], lvo = S.lam_out_v[i];
		// p' = p + v'' dt, v'' = v' + C dt / 80
		const float2 lvn = add2(lvo, mul2(lp, dt));
		// per-lane partial adjoints, warp-summed at the end (lane 0 holds the
		// agent's own terms)
		float2 lpi = lane == 0 ? lp : v2(0, 0), lvi = v2(0, 0);
		const float2 lC = mul2(lvn, dt / 80.0f);
		// preferred velocity (agent.cpp:52-59)
		const float2 w = sub2(A.goal, A.pos);
		const bool at_goal = dot2(w, w) <= A.radius * A.radius;
		A.pref = at_goal ? v2(0, 0) : vmul(vnorm(w), A.prefspeed);
		const bool moving = !viszero(A.pref);
		const int K = S.tape_cnt[i];
		const uint32_t* list = S.tape_list + (size_t)i * S.maxnb;
		// a = sum coeff F / m (ForceBasedFunction::GetGradient with
		// policy.cpp:78-89); the forward step recorded a before the clamp
		float2 la = v2(0, 0);
		if (moving) {
			const float2 a = S.tape_acc[i];
			const float2 ac = vclamp(a, A.maxacc);
			const float2 u = add2(A.vel, mul2(ac, dt));
			const float2 lu = clamp_adj(u, A.maxspeed, lvn);
			if (lane == 0) lvi = add2(lvi, lu);
			la = clamp_adj(a, A.maxacc, mul2(lu, dt));
		}
		float2 lpref = v2(0, 0);
		float dV0 = 0, dsig = 0, dk = 0, dtau0 = 0;
		for (int c = 0; c < pol.ncost; ++c) {
			const CostDesc& cd = pol.cost[c];
			if (cd.kind == K_GOALREACHING && lane == 0) {
				const float2 lF = mul2(la, cd.coeff / cd.p[5]);
				const float mr = fmaxr(A.relax, dt);
				lpref = add2(lpref, mul2(lF, 1.0f / mr));
				lvi = sub2(lvi, mul2(lF, 1.0f / mr));
			}
		}
		const bool contact = pol.contact_scale > 0;
		if (moving || contact) {
			for (int k = lane; k < K; k += 32) {
				const uint32_t e = list[k];
				const int j = (int)(e & 0x0FFFFFFFu);
				const float2 pj = add2(S.a_pos[j], group_offset(e >> 28, sd.width, sd.height));
				const float2 D = sub2(A.pos, pj);
				const float d2 = dot2(D, D);
				const float rj = S.prm[j].x;
				float2 lpj = v2(0, 0), lvj = v2(0, 0);
				if (moving) {
					const float2 vj = S.a_vel[j];
					const float4 nb = S.adj_nb[j];
					for (int c = 0; c < pol.ncost; ++c) {
						const CostDesc& cd = pol.cost[c];
						if (cd.kind == K_GOALREACHING || d2 > cd.range * cd.range) continue;
						const float2 lF = mul2(la, cd.coeff / cd.p[5]);
						if (cd.kind == K_SOCIALFORCES) {
							const float2 ebj = v2(nb.x, nb.y);
							const SfAdj r = sf_pair_adj(A, cd, pj, vj, ebj, rj, lF);
							lpi = add2(lpi, r.lR);
							lpj = sub2(lpj, r.lR);
							lvj = add2(lvj, r.lvj);
							// Eb_j = (g_j - p_j)/|g_j - p_j| away from the goal
							lpj = sub2(lpj, mul2(sub2(r.lEb, mul2(ebj, dot2(ebj, r.lEb))), nb.z));
							dV0 += r.lV0;
							dsig += r.lsigma;
						} else {
							const PlAdj r = pl_pair_adj(A, cd, pj, vj, rj, lF);
							lpi = add2(lpi, r.lx);
							lpj = sub2(lpj, r.lx);
							lvi = add2(lvi, r.lv);
							lvj = sub2(lvj, r.lv);
							dk += r.lk;
							dtau0 += r.ltau0;
						}
					}
				}
				// contact forces (all neighbours): C = sum scale (rsum - |D|) D/|D|
				if (contact) {
					const float2 lD = contact_adj(D, A.radius + rj, pol.contact_scale, lC);
					lpi = add2(lpi, lD);
					lpj = sub2(lpj, lD);
				}
				if (lpj.x != 0) atomicAdd(&S.lam_in_p[j].x, lpj.x);
				if (lpj.y != 0) atomicAdd(&S.lam_in_p[j].y, lpj.y);
				if (lvj.x != 0) atomicAdd(&S.lam_in_v[j].x, lvj.x);
				if (lvj.y != 0) atomicAdd(&S.lam_in_v[j].y, lvj.y);
			}
		}
		// static obstacle edges (the list recomputed from the state the step
		// started from, as the forward step gathered it): SocialForces
		// obstacle forces (compute_force) and contact with edges
		if (OBST && sd.nedges > 0 && (moving || contact))
			lpi = add2(lpi, obstacle_adjoint(S, sd, pol, A, gw, lane, moving, contact, la, lC));
		// warp sums (lane 0 also holds the goal-force terms)
		float vals[8] = { lpi.x, lpi.y, lvi.x, lvi.y, dV0, dsig, dk, dtau0 };
		for (int q = 0; q < 8; ++q)
			for (int o = 16; o > 0; o >>= 1) vals[q] += __shfl_xor_sync(0xffffffffu, vals[q], o);
		if (lane == 0) {
			float2 P = v2(vals[0], vals[1]);
			if (!at_goal) P = sub2(P, mul2(normalize_adj(w, lpref), A.prefspeed));   // pref = s (g - p)/|g - p|
			atomicAdd(&S.lam_in_p[i].x, P.x); atomicAdd(&S.lam_in_p[i].y, P.y);
			atomicAdd(&S.lam_in_v[i].x, vals[2]); atomicAdd(&S.lam_in_v[i].y, vals[3]);
			float* dp = S.dparams + 4 * sc;
			if (vals[4] != 0) atomicAdd(dp + 0, vals[4]);
			if (vals[5] != 0) atomicAdd(dp + 1, vals[5]);
			if (vals[6] != 0) atomicAdd(dp + 2, vals[6]);
			if (vals[7] != 0) atomicAdd(dp + 3, vals[7]);
		}
		__syncwarp();
	}
}

// loss += w |p - target|^2 summed over agents (double accumulation)
__global__ void k_loss(DevState S, const float2* target, float w, double* loss)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	float v = 0;
	if (i < S.n) {
		const float2 d = sub2(S.pos[i], target[i]);
		v = w * dot2(d, d);
	}
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(loss, (double)v);
}

// lam_p = lam_p_in + 2 w (pos - target); lam_v = lam_v_in
__global__ void k_inject(int n, const float2* pos, const float2* target, float w, const float2* lpin,
                         const float2* lvin, float2* lpout, float2* lvout)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float2 d = sub2(pos[i], target[i]);
	lpout[i] = add2(lpin[i], mul2(d, 2 * w));
	lvout[i] = lvin[i];
}

}  // namespace umans
