// the fused per-agent step (k_agent)
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// ------------------------------------------------------------------------
// the fused per-agent step
// ------------------------------------------------------------------------
// MODE 0: any policy.  MODE 1: every policy has force-based costs only
// (SocialForcesAvoidance, PowerLaw, GoalReachingForce), whatever its method
// (the velocity comes from the cost targets, finish_forces); the generic
// sampling, ORCA and finite-difference code is compiled out, which lowers
// register use and raises occupancy.
// TAPE: also record the neighbour lists and the pre-clamp acceleration for
// the differentiable form's backward pass
// OBST: the obstacle-edge gather compiled in (the force-only kernel of
// obstacle-free groups leaves it out, which keeps its registers)

// MODE 2: every policy is the global method with one ORCA cost (the ORCA
// solve only: 64 registers, 8 blocks per SM, against 128 and 4 for MODE 0).
// MODE 3: every policy samples a regular schedule with one Karamouzas cost
// (the general sampler compiled out: 21% faster than MODE 0 on a 100k-agent
// corridor at the same 128 registers; at 96 registers it spilled and was
// slower).
// SMEM_LINES: the ORCA lines and their projections (the Karamouzas
// sampler's scratch) in shared memory after the lists, 16-byte aligned,
// instead of the global line scratch
template <int MODE, bool TAPE, bool OBST, bool SAMP, bool SMEM_LINES = false>
__device__ __forceinline__ void agent_pass(const DevState& S, int dump)
{
	extern __shared__ unsigned char smem[];
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
	const int maxnb = S.maxnb;
	uint32_t* base = reinterpret_cast<uint32_t*>(smem) + (size_t)wib * 4 * maxnb;
	WarpLists L{ base, reinterpret_cast<float*>(base + maxnb), reinterpret_cast<int*>(base + 2 * maxnb),
	             reinterpret_cast<float*>(base + 3 * maxnb) };
	bool overflow = false;
	if constexpr (MODE == 1) {
		float* stash = reinterpret_cast<float*>(smem) + (size_t)(blockDim.x >> 5) * 4 * maxnb + wib * 32 * STASH_STRIDE;
		force_agents<TAPE, OBST, SAMP>(S, L, stash, lane, gw, &overflow);
		if (overflow && lane == 0) atomicOr(S.status, ST_NEIGHBOUR_OVERFLOW);
		return;
	}
	float* fx = reinterpret_cast<float*>(L.nid);   // per-neighbour terms
	float* fy = L.aux;
	float4* lines;
	if constexpr (SMEM_LINES) {
		const uintptr_t l0 = reinterpret_cast<uintptr_t>(smem + (size_t)(blockDim.x >> 5) * 16 * maxnb);
		lines = reinterpret_cast<float4*>((l0 + 15) & ~(uintptr_t)15) + (size_t)wib * 2 * maxnb;
	} else {
		lines = S.scratch + (size_t)gw * 2 * maxnb;
	}
	float4* proj = lines + maxnb;

	WorkIter w;
	const int n_items = S.t_end - S.t_begin;
	for (int it = work_first<8>(S, w, n_items, gw, lane); it >= 0; it = work_after<8>(S, w, it, lane, n_items)) {
		const int t = S.t_begin + it;
		const int slot = S.sSlot[t];
		const float4 sb = S.sB[t];
		const float4 prm = S.prm[slot];
		const int pi = S.pol[slot];
		const PolicyDesc& pol = S.pols[pi];
		AgentCtx A;
		A.pos = S.sP[t]; A.vel = S.sV[t]; A.pref = V(sb.x, sb.y); A.goal = S.goal[slot];
		A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
		const int sc = S.agent_scen[slot];
		const ScenDesc sd = S.scen[sc];
		const GridParams G = S.grid[sc];
		A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;

		const int K = gather(S, G, S.cell_base[sc], sd.world, sd.width, sd.height, L, t, A.pos, pol.range, lane, &overflow);
		NbView N;
		N.ref = L.ref; N.d2 = L.key; N.K = K; N.sP = S.sP; N.sV = S.sV; N.sB = S.sB; N.sE = S.sE;
		N.W = sd.width; N.H = sd.height;
		N.edges = S.edges; N.obs = nullptr; N.KO = 0;

		if (dump) {
			const int cap = S.dump_cap;
			for (int k = lane; k < K && k < cap; k += 32) {
				S.dump_ids[(size_t)slot * cap + k] = S.sId[L.ref[k] & 0x0FFFFFFFu];
				S.dump_d2[(size_t)slot * cap + k] = L.key[k];
			}
			if (lane == 0) S.dump_cnt[slot] = K;
			__syncwarp();
			continue;
		}
		if (TAPE) {
			for (int k = lane; k < K; k += 32) {
				const uint32_t rr = L.ref[k];
				S.tape_list[(size_t)slot * maxnb + k] = (rr & 0xF0000000u) | (uint32_t)S.sSlot[rr & 0x0FFFFFFFu];
			}
			if (lane == 0) S.tape_cnt[slot] = K;
		}
		if (OBST && sd.nedges > 0) {
			uint32_t* ol = S.obs_list + (size_t)gw * S.max_obs;
			N.KO = gather_obstacles(S, sd, A.pos, pol.range, lane, ol);
			N.obs = ol;
		}

		// phase 5: contact forces (policy.cpp:107-141), independent of phase 4
		float2 contact = V(0, 0);
		if (pol.contact_scale > 0) {
			for (int b0 = 0; b0 < K; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < K) {
					// d2[k] is |pos - neighbour|^2 computed exactly as vsq(diff); if it
					// exceeds (r + r_j)^2 by 1e-5 relative, sqrt(d2) >= r + r_j and the
					// overlap test below is false
					const float rsum = A.radius + nb_radius(N, k);
					if (!(N.d2[k] > rsum * rsum * 1.00001f)) {
						const float2 diff = vsub(A.pos, nb_pos(N, k));
						const float inter = rsum - vmag(diff);
						if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
					}
				}
				contact = ordered_accumulate(contact, f, take);
			}
			// colliding obstacle edges, after the agents (policy.cpp:126-137)
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

		// phase 4: Policy::ComputeNewVelocity (policy.cpp:43-76)
		float2 nv = V(0, 0);
		uint32_t rng_next = 0;
		bool rng_used = false;
		if (MODE == 2 && !viszero(A.pref)) {
			// global method, one ORCA cost: its solution (ORCA::GetGlobalMinimum)
			int nl = 0;
			const float2 best = orca_solve(A, N, pol.cost[0], lines, proj, &nl, lane);
			const float2 acc = vclamp(vdiv(vsub(best, A.vel), fmaxr(pol.relax_time, A.dt)), A.maxacc);
			nv = vclamp(vadd(A.vel, vmul(acc, A.dt)), A.maxspeed);
		} else if (MODE == 3 && !viszero(A.pref)) {
			// sampling a regular schedule with one Karamouzas cost
			CostPrep P;
			P.lines = lines; P.nlines = 0; P.orca_v = V(0, 0);
			karamouzas_prep(A, N, pol.cost[0], 0, lane, &P);
			const float2 best = sample_min<true>(S, A, N, pol, P, S.rng[slot], lane, lines, reinterpret_cast<float*>(proj));
			const float2 acc = vclamp(vdiv(vsub(best, A.vel), fmaxr(pol.relax_time, A.dt)), A.maxacc);
			nv = vclamp(vadd(A.vel, vmul(acc, A.dt)), A.maxspeed);
		} else if (MODE == 0 && !viszero(A.pref)) {
			CostPrep P;
			P.lines = lines; P.nlines = 0; P.orca_v = V(0, 0);
			for (int ci = 0; ci < pol.ncost; ++ci) {
				const CostDesc& c = pol.cost[ci];
				if (is_force_based(c.kind)) P.target[ci] = target_velocity(A, N, c, lane, fx, fy);
				else if (c.kind == K_KARAMOUZAS) karamouzas_prep(A, N, c, ci, lane, &P);
				else if (c.kind == K_ORCA) {
					P.orca_v = orca_solve(A, N, c, lines, proj, &P.nlines, lane);
				}
			}
			float2 acc;
			if (pol.method == M_GRADIENT) {
				// Policy::getAccelerationFromGradient: policy.cpp:78-89
				float2 T = V(0, 0);
				int grad_draws = 0;
				for (int ci = 0; ci < pol.ncost; ++ci) {
					const CostDesc& c = pol.cost[ci];
					float2 g;
					if (is_force_based(c.kind)) g = vdiv(vsub(A.vel, P.target[ci]), A.dt);
					else if (c.kind == K_RANDOM) {
						// RandomFunction::GetGradient (RandomFunction.cpp:30-33): two
						// numbers in [-1, 1]; the reference build evaluates the
						// constructor's second argument first
						const uint32_t r0 = S.rng[slot];
						const float gy = rng_uniform(mulmod(S.lcgpow[grad_draws + 1], r0), -1, 1);
						const float gx = rng_uniform(mulmod(S.lcgpow[grad_draws + 2], r0), -1, 1);
						grad_draws += 2;
						g = V(gx, gy);
					} else if (c.kind == K_GENERIC) g = V(0, 0);   // FD of a zero cost
					else if (c.kind == K_TTCADCA)
						g = grad_ttcadca(A, N, c, A.vel, lane, fx, fy, reinterpret_cast<float*>(proj));
					else if (c.kind == K_FOE) g = grad_foe(A, N, c, A.vel, lane, fx, fy);
					else if (c.kind >= K_PLUGIN0 &&
					         plugin_gradient(c.kind - K_PLUGIN0, A, N, c, A.vel, lane, fx, fy, &g)) {
						// the plugin's GetGradient
					} else {
						// CostFunction::GetGradient default: costFunction.cpp:36-54;
						// lanes 0..3 evaluate the four probes
						const float d = 0.1f;
						const int which = lane & 3;
						float2 probe = A.vel;
						if (which == 0) probe = vsub(A.vel, V(d, 0));
						else if (which == 1) probe = vadd(A.vel, V(d, 0));
						else if (which == 2) probe = vsub(A.vel, V(0, d));
						else probe = vadd(A.vel, V(0, d));
						const float cv = eval_cost(A, N, c, P, ci, probe);
						const float cl = __shfl_sync(0xffffffffu, cv, 0), cr = __shfl_sync(0xffffffffu, cv, 1);
						const float cb = __shfl_sync(0xffffffffu, cv, 2), ct = __shfl_sync(0xffffffffu, cv, 3);
						g = V((cr - cl) / (2 * d), (ct - cb) / (2 * d));
					}
					T = vadd(T, vmul(g, c.coeff));
				}
				acc = vmul(T, -1);
				if (TAPE && lane == 0) S.tape_acc[slot] = acc;
				if (grad_draws > 0) {
					rng_used = true;
					rng_next = mulmod(S.lcgpow[grad_draws], S.rng[slot]);
				}
			} else {
				float2 best;
				const CostDesc& c0 = pol.cost[0];
				if (pol.method == M_GLOBAL && pol.ncost == 1 && c0.kind == K_ORCA) best = P.orca_v;
				else if (pol.method == M_GLOBAL && pol.ncost == 1 && is_force_based(c0.kind)) best = P.target[0];
				else if (pol.method == M_GLOBAL && pol.ncost == 1 && c0.kind >= K_PLUGIN0 &&
				         plugin_global_minimum(c0.kind - K_PLUGIN0, A, N, c0, lane, &best)) {
					// the plugin's GetGlobalMinimum
				}
				else {
					const uint32_t r0 = S.rng[slot];
					best = sample_min(S, A, N, pol, P, r0, lane, lines, reinterpret_cast<float*>(proj));
					if (pol.draws > 0) {
						rng_used = true;
						rng_next = mulmod(S.lcgpow[pol.nsamples * pol.draws], r0);
					}
				}
				acc = vdiv(vsub(best, A.vel), fmaxr(pol.relax_time, A.dt));
			}
			acc = vclamp(acc, A.maxacc);
			nv = vclamp(vadd(A.vel, vmul(acc, A.dt)), A.maxspeed);
		}

		// phase 6: Agent::UpdateVelocityAndPosition (agent.cpp:71-93)
		if (lane == 0) {
			update_agent(S, sd, slot, A.pos, A.pref, A.dt, nv, contact);
			if (rng_used) S.rng[slot] = rng_next;
		}
		__syncwarp();
	}
	work_end(S, lane);
	if (overflow && lane == 0) atomicOr(S.status, ST_NEIGHBOUR_OVERFLOW);
}

template <int MODE, bool TAPE = false, bool OBST = true, bool SAMP = false>
__global__ void __launch_bounds__(128, MODE == 1 ? 8 : (MODE == 2 ? 8 : 4)) k_agent(DevState S, int dump)
{
	agent_pass<MODE, TAPE, OBST, SAMP>(S, dump);
}

// Small worlds (the range of build_small), several steps in one cooperative
// launch, so that a step costs no launch: block 0 builds the step's grid
// (build_small_smem) while the other blocks wait at a grid barrier, then every
// block updates its agents (one warp per agent where the launch has the
// warps, the ORCA lines in shared memory) and a second grid barrier ends
// the step.  S describes the launch as
// the agent pass's only one (t_begin 0, t_end n, total_warps the launch's
// warps, the interleaved schedule).  The fences of the grid barrier order the
// build's writes before every block's reads, and each step's agent writes
// before the next build.  After a step that set a status bit every block
// leaves the loop (all read the status after the same barrier): the host
// reports it, or re-runs the steps from its snapshot with a longer
// neighbour capacity.
constexpr int SMALL_STEPS_MAX_THREADS = 256;
template <int MODE>
__global__ void __launch_bounds__(SMALL_STEPS_MAX_THREADS, MODE == 2 ? 4 : 2) k_small_steps(DevState S, int nsteps)
{
	__shared__ SmallGrid B;
	for (int s = 0; s < nsteps; ++s) {
		if (blockIdx.x == 0) build_small_smem(S, B);
		grid_barrier(S);
		agent_pass<MODE, false, true, false, true>(S, 0);
		grid_barrier(S);
		if (__ldcg(S.status) != 0) break;
	}
}

}  // namespace umans
