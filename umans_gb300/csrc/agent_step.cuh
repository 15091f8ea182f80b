// pieces of the per-agent step shared by its kernels: the agent update,
// agent-to-warp schedules, the force-only policies' warp-per-agent path
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// ------------------------------------------------------------------------
// agent update
// ------------------------------------------------------------------------
// Agent::UpdateVelocityAndPosition (agent.cpp:71-93) for one agent: the
// contact force over the agent mass (80) added to the policy's velocity nv,
// the viewing direction, the new position (wrapped in toric worlds:
// worldToric.cpp:81-108).
__device__ __forceinline__ void update_agent(const DevState& S, const ScenDesc& sd, int slot, float2 pos,
                                             float2 pref, float dt, float2 nv, float2 contact)
{
	const float2 af = vdiv(contact, 80.0f);
	const float2 vel = vadd(nv, vmul(af, dt));
	const float2 vd = vdiv(vadd(vmul(vel, 2), pref), 3);
	// (double)|vd|^2 > 0.01 <=> |vd|^2 > 0.01f (0.01f is the float just below 0.01)
	if (vsq(vd) > 0.01f) S.view[slot] = vnorm(vd);
	float2 p = vadd(pos, vmul(vel, dt));
	if (sd.world == W_TORIC) {
		const float hw = 0.5f * sd.width, hh = 0.5f * sd.height;
		float x = p.x, y = p.y;
		if (x > hw) x -= sd.width;
		else if (x < -hw) x += sd.width;
		if (y > hh) y -= sd.height;
		else if (y < -hh) y += sd.height;
		p = V(x, y);
	}
	S.pos[slot] = p;
	S.vel[slot] = vel;
	S.vwf[slot] = nv;
}

// ------------------------------------------------------------------------
// agents to warps
// ------------------------------------------------------------------------
// Items [0, n) (agents, or groups of four agents) handed to the warps of a
// launch.  Schedule 0: warp w takes w, w + W, w + 2W, ... (W warps).
// Schedule 1: warp w a contiguous range.  Schedule 2, a work list: tiles of
// TILE items, each warp taking the next tile from the launch's counter
// when it has finished one; work_end then counts the warp out, and the last
// warp to finish resets the counter for the next launch (no warp waits).
struct WorkIter {
	int end, step;
};
// (WL false: the launch never uses the work list; its code is left out)
template <int TILE, bool WL>
__device__ __forceinline__ int work_take(const DevState& S, WorkIter& w, int lane, int n)
{
	unsigned k = 0;
	if (lane == 0) k = atomicAdd(S.work, 1u);
	k = __shfl_sync(0xffffffffu, k, 0);
	const long long b = (long long)k * TILE;
	if (b >= n) return -1;
	w.end = (int)min((long long)n, b + TILE);
	w.step = 1;
	return (int)b;
}
// the first item of the warp, the same on every lane; -1 when none
template <int TILE, bool WL = true>
__device__ __forceinline__ int work_first(const DevState& S, WorkIter& w, int n, int gw, int lane)
{
	if (WL && S.sched == 2) return work_take<TILE, WL>(S, w, lane, n);
	int i;
	if (S.sched == 1) {
		const int per = (n + S.total_warps - 1) / S.total_warps;
		i = gw * per; w.end = min(n, i + per); w.step = 1;
	} else { i = gw; w.end = n; w.step = S.total_warps; }
	return i < w.end ? i : -1;
}
// the item after i; -1 when none is left
template <int TILE, bool WL = true>
__device__ __forceinline__ int work_after(const DevState& S, WorkIter& w, int i, int lane, int n)
{
	i += w.step;
	if (i < w.end) return i;
	if (!WL || S.sched != 2) return -1;
	return work_take<TILE, WL>(S, w, lane, n);
}
template <bool WL = true>
__device__ __forceinline__ void work_end(const DevState& S, int lane)
{
	if (!WL || S.sched != 2 || lane != 0) return;
	const unsigned d = atomicAdd(S.work + 1, 1u);
	if (d == (unsigned)S.total_warps - 1u) {   // every warp has taken its last ticket
		S.work[0] = 0u;
		S.work[1] = 0u;
	}
}

// ------------------------------------------------------------------------
// force-only policies
// ------------------------------------------------------------------------
// Policies whose costs are all force-based (SocialForces, PowerLaw,
// GoalReaching), whatever their method, take this path.  Per agent the warp
// gathers the neighbour list and evaluates the neighbour terms: pair forces
// and contact forces in one pass over the list, each summed in list order.
// The per-agent remainder (GoalReachingForce, the cost targets and the
// method's choice of velocity, the clamps, Agent::UpdateVelocityAndPosition)
// then runs for up to 32 agents at once, one per lane, from a per-warp
// record in shared memory: t, the force of each cost (x, y), the contact
// force (x, y).  The stride is odd, so lane j's record starts in bank j.
constexpr int STASH_STRIDE = 2 + 2 * MAX_COSTS + 1;

// The neighbour force of cost c (SocialForces or PowerLaw; agents, then
// obstacle edges), as compute_force.  With contact_scale > 0 the same pass
// over the list also forms the agents' contact forces (policy.cpp:107-125)
// and sums them in list order into *contact.
__device__ float2 force_and_contact(const AgentCtx& A, const NbView& N, const CostDesc& c, float contact_scale,
                                    int lane, float* fx, float* fy, float2* contact)
{
	const float rs = c.range * c.range;
	const bool sf = c.kind == K_SOCIALFORCES;
	const SfConst SK = sf_const(A, c);
	float2 cacc = V(0, 0);
	for (int b0 = 0; b0 < N.K; b0 += 32) {
		const int k = b0 + lane;
		bool take = false;
		float2 fc = V(0, 0);
		if (k < N.K) {
			const float2 np = nb_pos(N, k);
			const float nr = nb_radius(N, k);
			const float d2 = N.d2[k];
			float2 f = V(0, 0);
			if (d2 <= rs) f = sf ? sf_force(A, SK, np, nb_E(N, k), nr) : pl_force(A, c, np, nb_vel(N, k), nr);
			fx[k] = f.x;
			fy[k] = f.y;
			if (contact_scale > 0) {
				// d2 is |pos - neighbour|^2 computed exactly as vsq(diff); if it
				// exceeds (r + r_j)^2 by 1e-5 relative, sqrt(d2) >= r + r_j and
				// the overlap test is false
				const float rsum = A.radius + nr;
				if (!(d2 > rsum * rsum * 1.00001f)) {
					const float2 diff = vsub(A.pos, np);
					const float inter = rsum - vmag(diff);
					if (inter > 0) { take = true; fc = vmul(vnorm(diff), contact_scale * inter); }
				}
			}
		}
		if (contact_scale > 0) cacc = ordered_accumulate(cacc, fc, take);
	}
	if (contact_scale > 0) *contact = cacc;
	__syncwarp();
	const float2 sum = list_sum(fx, fy, N.K, lane);
	__syncwarp();
	return vadd(sum, obstacle_force(A, N, c, lane));
}

// Karamouzas's per-agent terms (Karamouzas.cpp: the time to collision at the
// preferred velocity, its deviation window): the time is a min, so lanes
// split the neighbours.
__device__ __forceinline__ void karamouzas_prep(const AgentCtx& A, const NbView& N, const CostDesc& c, int ci,
                                                int lane, CostPrep* P)
{
	float m = MAXF;
	const float md2 = c.range * c.range;
	for (int k = lane; k < N.K; k += 32) {
		if (N.d2[k] > md2) continue;
		const float tt = ttc_pair(A.pos, A.pref, A.radius, nb_pos(N, k), nb_vel(N, k), nb_radius(N, k));
		if (tt == 0) continue;
		if (tt < m) m = tt;
	}
	for (int k = lane; k < N.KO; k += 32) {
		float2 a, b;
		nb_seg(N, k, &a, &b);
		if (dist2_to_segment(A.pos, a, b) > md2) continue;
		const float tt = ttc_segment(A.pos, A.pref, A.radius, a, b);
		if (tt == 0) continue;
		if (tt < m) m = tt;
	}
	for (int o = 16; o > 0; o >>= 1) {
		const float x = __shfl_xor_sync(0xffffffffu, m, o);
		if (x < m) m = x;
	}
	P->ttcp[ci] = m;
	P->maxdev[ci] = karamouzas_maxdev(m);
	P->cosdev[ci] = cosf(P->maxdev[ci]);
}

// Candidate velocity i of a sampling policy (costFunction.cpp:99-158): the
// regular schedule from its table, or random sampling with the agent's
// minstd_rand0 stream jumped ahead to the sample's draws.
__device__ __forceinline__ float2 sample_velocity(const DevState& S, const PolicyDesc& pol, float2 base, float2 dir,
                                                  float dL, float radius, uint32_t rng0, int i)
{
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

// The remainder of a batch of nb agents, lane j taking record j.  The
// policy's method picks the new velocity from the cost targets
// (ForceBasedFunction::ComputeTargetVelocity, ForceBasedFunction.cpp:48-52):
// - gradient: the gradient step of policy.cpp:78-89;
// - global with one cost: its target, the cost's global minimum
//   (ForceBasedFunction::GetGlobalMinimum);
// - sampling, or global with several costs (the default schedule of
//   SamplingParameters::ApproximateGlobalOptimization): the first sample of
//   least summed cost 0.5 |v - target|^2 / dt (ForceBasedFunction.cpp:26-30,
//   costFunction.cpp:60-95), one lane running the agent's samples in order.
// SAMP false: every policy of the group uses the gradient method (the
// other methods' code is compiled out).
template <bool TAPE, bool SAMP>
__device__ void finish_forces(const DevState& S, const float* stash, int nb, int lane)
{
	if (lane >= nb) return;
	const float* rec = stash + lane * STASH_STRIDE;
	const int t = __float_as_int(rec[0]);
	const int slot = S.sSlot[t];
	const float4 sb = S.sB[t];
	const float4 prm = S.prm[slot];
	const PolicyDesc& pol = S.pols[S.pol[slot]];
	const ScenDesc& sd = S.scen[S.agent_scen[slot]];
	const float2 pos = S.sP[t], vel = S.sV[t], pref = V(sb.x, sb.y);
	const float dt = sd.dt;
	float2 nv = V(0, 0);
	if (!viszero(pref)) {
		float2 acc;
		if (!SAMP || pol.method == M_GRADIENT) {
			float2 T = V(0, 0);
			for (int ci = 0; ci < pol.ncost; ++ci) {
				const CostDesc& c = pol.cost[ci];
				const float2 F = c.kind == K_GOALREACHING ? vdiv(vsub(pref, vel), fmaxr(pol.relax_time, dt))
				                                          : V(rec[1 + 2 * ci], rec[2 + 2 * ci]);
				const float2 target = vadd(vel, vmul(vdiv(F, c.p[5]), dt));
				T = vadd(T, vmul(vdiv(vsub(vel, target), dt), c.coeff));
			}
			acc = vmul(T, -1);
			if (TAPE) S.tape_acc[slot] = acc;
		} else {
			float2 tg[MAX_COSTS];
#pragma unroll
			for (int ci = 0; ci < MAX_COSTS; ++ci) {
				if (ci >= pol.ncost) break;
				const CostDesc& c = pol.cost[ci];
				const float2 F = c.kind == K_GOALREACHING ? vdiv(vsub(pref, vel), fmaxr(pol.relax_time, dt))
				                                          : V(rec[1 + 2 * ci], rec[2 + 2 * ci]);
				tg[ci] = vadd(vel, vmul(vdiv(F, c.p[5]), dt));
			}
			float2 best = V(0, 0);
			if (!pol.use_sampling) {
				best = tg[0];
			} else {
				// sample_min's schedule (base, direction, length step)
				float2 base = V(0, 0);
				if (pol.table_base == 1) base = vel;
				float radius;
				if (pol.table_radius == 0) radius = prm.y;
				else if (pol.table_radius == 1) radius = prm.z;
				else radius = fminr(2.0f * prm.z, prm.w * dt);
				float2 dir = V(1, 0);
				if (pol.table_dir == 1) dir = vnorm(vel);
				else if (pol.table_dir == 2) dir = vnorm(pref);
				const float dL = radius / (float)pol.len_divisor;
				const uint32_t r0 = S.rng[slot];
				float bestC = MAXF;
				int bestI = -1;
				for (int i = 0; i < pol.nsamples; ++i) {
					const float2 v = sample_velocity(S, pol, base, dir, dL, radius, r0, i);
					float tc = 0;
#pragma unroll
					for (int ci = 0; ci < MAX_COSTS; ++ci) {
						if (ci >= pol.ncost) break;
						tc += pol.cost[ci].coeff * (0.5f * vsq(vsub(v, tg[ci])) / dt);
					}
					if (tc < bestC) { bestC = tc; bestI = i; }
				}
				if (bestI >= 0) best = sample_velocity(S, pol, base, dir, dL, radius, r0, bestI);
				if (pol.draws > 0) S.rng[slot] = mulmod(S.lcgpow[pol.nsamples * pol.draws], r0);
			}
			acc = vdiv(vsub(best, vel), fmaxr(pol.relax_time, dt));
		}
		acc = vclamp(acc, prm.w);
		nv = vclamp(vadd(vel, vmul(acc, dt)), prm.z);
	}
	update_agent(S, sd, slot, pos, pref, dt, nv, V(rec[2 * MAX_COSTS + 1], rec[2 * MAX_COSTS + 2]));
}

template <bool TAPE, bool OBST, bool SAMP>
__device__ void force_agents(const DevState& S, const WarpLists& L, float* stash, int lane, int gw, bool* overflow)
{
	float* fx = reinterpret_cast<float*>(L.nid);
	float* fy = L.aux;
	WorkIter w;
	const int n_items = S.t_end - S.t_begin;
	int nb = 0;
	for (int it = work_first<32>(S, w, n_items, gw, lane); it >= 0; it = work_after<32>(S, w, it, lane, n_items)) {
		const int t = S.t_begin + it;
		const int slot = S.sSlot[t];
		const float4 sb = S.sB[t];
		const float4 prm = S.prm[slot];
		const PolicyDesc& pol = S.pols[S.pol[slot]];
		AgentCtx A;
		A.pos = S.sP[t]; A.vel = S.sV[t]; A.pref = V(sb.x, sb.y); A.goal = V(0, 0);
		A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
		const int sc = S.agent_scen[slot];
		const ScenDesc sd = S.scen[sc];
		const GridParams G = S.grid[sc];
		A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;

		const int K = gather(S, G, S.cell_base[sc], sd.world, sd.width, sd.height, L, t, A.pos, pol.range, lane, overflow);
		NbView N;
		N.ref = L.ref; N.d2 = L.key; N.K = K; N.sP = S.sP; N.sV = S.sV; N.sB = S.sB; N.sE = S.sE;
		N.W = sd.width; N.H = sd.height;
		N.edges = S.edges; N.obs = nullptr; N.KO = 0;
		if (TAPE) {
			for (int k = lane; k < K; k += 32) {
				const uint32_t rr = L.ref[k];
				S.tape_list[(size_t)slot * S.maxnb + k] = (rr & 0xF0000000u) | (uint32_t)S.sSlot[rr & 0x0FFFFFFFu];
			}
			if (lane == 0) S.tape_cnt[slot] = K;
		}
		if (OBST && sd.nedges > 0) {
			uint32_t* ol = S.obs_list + (size_t)gw * S.max_obs;
			N.KO = gather_obstacles(S, sd, A.pos, pol.range, lane, ol);
			N.obs = ol;
		}

		float* rec = stash + nb * STASH_STRIDE;
		float2 contact = V(0, 0);
		bool contact_done = !(pol.contact_scale > 0);
		if (!viszero(A.pref)) {
			for (int ci = 0; ci < pol.ncost; ++ci) {
				const CostDesc& c = pol.cost[ci];
				if (c.kind == K_GOALREACHING) continue;
				const float2 f = force_and_contact(A, N, c, contact_done ? 0.0f : pol.contact_scale, lane, fx, fy,
				                                   &contact);
				contact_done = true;
				if (lane == 0) { rec[1 + 2 * ci] = f.x; rec[2 + 2 * ci] = f.y; }
			}
		}
		// contact forces (policy.cpp:107-141): the agents, when no cost pass
		// formed them, then the colliding obstacle edges
		if (!contact_done) {
			for (int b0 = 0; b0 < K; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < K) {
					const float rsum = A.radius + nb_radius(N, k);
					if (!(N.d2[k] > rsum * rsum * 1.00001f)) {
						const float2 diff = vsub(A.pos, nb_pos(N, k));
						const float inter = rsum - vmag(diff);
						if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
					}
				}
				contact = ordered_accumulate(contact, f, take);
			}
		}
		if (OBST && pol.contact_scale > 0) {
			for (int b0 = 0; b0 < N.KO; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < N.KO) {
					float2 a, b;
					nb_seg(N, k, &a, &b);
					const float2 diff = vsub(A.pos, nearest_on_segment(A.pos, a, b));
					const float inter = A.radius - vmag(diff);
					if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
				}
				contact = ordered_accumulate(contact, f, take);
			}
		}
		if (lane == 0) {
			rec[0] = __int_as_float(t);
			rec[2 * MAX_COSTS + 1] = contact.x;
			rec[2 * MAX_COSTS + 2] = contact.y;
		}
		if (++nb == 32) {
			__syncwarp();
			finish_forces<TAPE, SAMP>(S, stash, nb, lane);
			__syncwarp();
			nb = 0;
		}
	}
	if (nb > 0) {
		__syncwarp();
		finish_forces<TAPE, SAMP>(S, stash, nb, lane);
	}
	work_end(S, lane);
}

}  // namespace umans
