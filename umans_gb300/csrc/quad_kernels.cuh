// force-only policies, four agents per warp (k_force_quad)
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// ------------------------------------------------------------------------
// force-only policies, four agents per warp
// ------------------------------------------------------------------------
// force_agents with eight lanes per agent: four agents per warp, consecutive
// in cell order (so that their lists have similar lengths).  Every loop runs
// warp-uniformly to the largest of the four agents' trip counts, each
// agent's lanes predicated on their own; shuffles stay within an agent's
// eight lanes (width 8) and each agent takes its byte of a ballot.  An
// agent's list is two arrays in shared memory (reference, key); the force
// pass overwrites each entry in place with its force terms (x over the key,
// y over the reference).  Worlds without obstacle edges whose policies have
// at most one neighbour cost (SocialForces or PowerLaw) take this path.
constexpr int QG = 8, QN = 32 / QG;

struct QLane {
	int sg, sl;        // agent of this lane in the warp, lane within the agent
	int shift;         // QG * sg
	unsigned below;    // the agent's lanes below this one
};
__device__ __forceinline__ unsigned q_ballot(bool p, const QLane& q)
{
	return (__ballot_sync(0xffffffffu, p) >> q.shift) & 0xFFu;
}
template <class T>
__device__ __forceinline__ T q_shfl(T v, int src) { return __shfl_sync(0xffffffffu, v, src, QG); }
__device__ __forceinline__ int q_max(int v) { return __reduce_max_sync(0xffffffffu, v); }

// warp_sort_regs for a group of G lanes (sl: the lane in the group): P = G M
// <= 64 packed keys, M per lane; entry i = G m + sl.  Exchanges at distances
// of G and more are between a lane's own registers.  The sorted keys also
// give the near-tie flags of fix_near_ties (pair (i, i+1) within the relative
// window win): every lane of the group returns the first and last flagged
// pair in *f0, *f1 (*f0 > *f1 when none is flagged).
template <int G, int M>
__device__ __forceinline__ void group_sort_regs(const WarpLists& L, int s, int len, int sl, float win, int* f0,
                                                int* f1)
{
	constexpr int QG = G;
	struct { int sl; } q{ sl };
	constexpr int P = QG * M;
	static_assert(P <= 64, "positions take at most 6 bits");
	constexpr int PB = P <= 32 ? 5 : 6;
	constexpr uint32_t PMASK = (1u << PB) - 1u;
	uint32_t u[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		u[m] = (i < len) ? ((__float_as_uint(L.key[s + i]) & ~PMASK) | (uint32_t)i) : 0xffffffffu;
	}
#pragma unroll
	for (int size = 2; size <= P; size <<= 1) {
#pragma unroll
		for (int j = size >> 1; j > 0; j >>= 1) {
#pragma unroll
			for (int m = 0; m < M; ++m) {
				const int i = m * QG + q.sl;
				const bool up = (i & size) == 0;
				if (j >= QG) {
					const int mm = m ^ (j / QG);
					if (mm > m) {
						const uint32_t a = u[m], b = u[mm];
						if (up ? (a > b) : (a < b)) { u[m] = b; u[mm] = a; }
					}
				} else {
					const uint32_t o = __shfl_xor_sync(0xffffffffu, u[m], j, QG);
					const bool lower = (q.sl & j) == 0;
					u[m] = (lower == up) ? min(u[m], o) : max(u[m], o);
				}
			}
		}
	}
	float k[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		const int from = s + (int)(u[m] & PMASK);
		k[m] = (i < len) ? L.key[from] : 0.0f;
		u[m] = (i < len) ? L.ref[from] : 0u;
	}
	__syncwarp();
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		if (i < len) {
			L.ref[s + i] = u[m];
			L.key[s + i] = k[m];
		}
	}
	int lo = 0x7fffffff, hi = -1;
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		// the key of entry i + 1: the next lane's, or lane 0's next register
		const float a = __shfl_down_sync(0xffffffffu, k[m], 1, QG);
		const float b = __shfl_sync(0xffffffffu, k[m + 1 < M ? m + 1 : m], 0, QG);
		const float nx = q.sl < QG - 1 ? a : b;
		if (i + 1 < len && nx - k[m] <= win * nx) { lo = min(lo, i); hi = max(hi, i); }
	}
#pragma unroll
	for (int o = 1; o < QG; o <<= 1) {
		lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o, QG));
		hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o, QG));
	}
	*f0 = lo;
	*f1 = hi;
	__syncwarp();
}

// warp_sort (bitonic in shared memory, by (key, id)) for an agent's eight
// lanes; the network is sized for the longest of the four lists.
__device__ void q_sort_smem(const DevState& S, const WarpLists& L, int s, int len, int netlen, const QLane& q)
{
	if (netlen <= 1) return;
	int lp = 0;
	while ((1 << lp) < netlen) ++lp;
	const int halfP = 1 << (lp - 1);
	for (int ls = 1; ls <= lp; ++ls) {
		const int lh = ls - 1;
		for (int k = q.sl; k < halfP; k += QG) {
			const int blk = k >> lh, pos = k & ((1 << lh) - 1);
			const int lo = (blk << ls) + pos, hi = (blk << ls) + (1 << ls) - 1 - pos;
			if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
		}
		__syncwarp();
		for (int lj = lh - 1; lj >= 0; --lj) {
			for (int k = q.sl; k < halfP; k += QG) {
				const int lo = ((k >> lj) << (lj + 1)) | (k & ((1 << lj) - 1)), hi = lo + (1 << lj);
				if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
			}
			__syncwarp();
		}
	}
}

// The first and last pair (i, i+1) of the agent's sorted list [s, e) whose
// keys are within the relative window win (as fix_near_ties; *f0 > *f1 when
// none), on every lane of the agent.
__device__ void q_near_ties(const WarpLists& L, int s, int e, const QLane& q, float win, int* f0, int* f1)
{
	const int npairs = e - 1 - s;
	const int pmax = q_max(npairs);
	int lo = 0x7fffffff, hi = -1;
	for (int b = 0; b < pmax; b += QG) {
		const int i = b + q.sl;
		if (i < npairs) {
			const float a = L.key[s + i], c = L.key[s + i + 1];
			if (c - a <= win * c) { lo = min(lo, i); hi = max(hi, i); }
		}
	}
#pragma unroll
	for (int o = 1; o < QG; o <<= 1) {
		lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o, QG));
		hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o, QG));
	}
	*f0 = lo;
	*f1 = hi;
}

// fix_near_ties for an agent's eight lanes, given its first and last flagged
// pairs f0 <= f1 (relative to s): the agent's first lane walks the pairs
// between them and re-sorts each run of near-equal keys in the reference's
// order (runs are disjoint, and re-sorting one changes no flag of the pairs
// after it).
__device__ void q_fix_near_ties(const DevState& S, const WarpLists& L, int s, int f0, int f1, float2 qp,
                                const QLane& q, float win)
{
	if (!__any_sync(0xffffffffu, f0 <= f1)) return;
	__syncwarp();
	if (f0 <= f1 && q.sl == 0) {
		int k = s + f0;
		const int kend = s + f1;   // the last flagged pair
		while (k <= kend) {
			const float a = L.key[k], c = L.key[k + 1];
			if (c - a <= win * c) {
				const int r0 = k;
				++k;
				while (k <= kend) {
					const float a2 = L.key[k], c2 = L.key[k + 1];
					if (!(c2 - a2 <= win * c2)) break;
					++k;
				}
				sort_run(S, L, r0, k, qp);   // pairs r0 .. k-1 flagged: entries r0 .. k
			}
			++k;
		}
	}
	__syncwarp();
}

// gather for an agent's eight lanes (live false: an empty list).
__device__ int q_gather(const DevState& S, const GridParams& G, int cb, int world, float W, float H,
                        const WarpLists& L, int t, float2 p, float r, bool live, const QLane& q, bool* overflow)
{
	int K = 0, K0 = 0;
	const int maxnb = S.maxnb;
	live = live && r > 0;   // dist < r*r never holds for r = 0
	const float r2 = r * r;
	const double r2d = (double)r2;
	const float r2lo = r2 * 0.999999f, r2hi = r2 * 1.000001f;
	for (int g = 0; g < 5; ++g) {
		float2 disp = V(0, 0);
		bool active = live;
		if (g > 0) {
			// worldToric.cpp:64-76 (see gather)
			if (world != W_TORIC) active = false;
			else if (g == 1) { active = active && (p.x - r) < -0.5f * W; disp = V(W, 0); }
			else if (g == 2) { active = active && (p.x + r) > 0.5f * W; disp = V(-W, 0); }
			else if (g == 3) { active = active && (p.y - r) < -0.5f * H; disp = V(0, H); }
			else { active = active && (p.y + r) > 0.5f * H; disp = V(0, -H); }
		}
		if (__any_sync(0xffffffffu, active)) {
			const float2 qp = vadd(p, disp);
			const int gs = K;
			int cx0 = 0, cx1 = -1, cy0 = 0, nrows = 0;
			if (active) {
				cx0 = cell_coord((qp.x - r - G.x0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.nx);
				cx1 = cell_coord((qp.x + r - G.x0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.nx);
				cy0 = cell_coord((qp.y - r - G.y0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.ny);
				const int cy1 = cell_coord((qp.y + r - G.y0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.ny);
				nrows = cy1 - cy0 + 1;
			}
			const int maxrows = q_max(nrows);
			// QG rows at a time: lane k loads the sorted range of row k, the rows
			// are concatenated and scanned two chunks of QG candidates per pass
			for (int r0 = 0; r0 < maxrows; r0 += QG) {
				const int nr = nrows - r0;
				int rs = 0, len = 0;
				if (q.sl < nr) {
					const int c0 = cb + (cy0 + r0 + q.sl) * G.nx;
					rs = S.start[c0 + cx0];
					len = S.start[c0 + cx1 + 1] - rs;
				}
				int incl = len;
#pragma unroll
				for (int o = 1; o < QG; o <<= 1) {
					const int v = __shfl_up_sync(0xffffffffu, incl, o, QG);
					if (q.sl >= o) incl += v;
				}
				const int beg = incl - len;
				const int total = q_shfl(incl, QG - 1);
				const int maxtotal = q_max(total);
				for (int base = 0; base < maxtotal; base += 2 * QG) {
					const int nh = base + QG < maxtotal ? 2 : 1;
					int tt[2];
					float2 cp[2];
#pragma unroll
					for (int h = 0; h < 2; ++h) {
						if (h >= nh) break;
						const int c = base + QG * h + q.sl;
						int rr = 0;
#pragma unroll
						for (int step = QG / 2; step > 0; step >>= 1)
							if (q_shfl(beg, rr + step) <= c) rr += step;
						tt[h] = q_shfl(rs, rr) + (c - q_shfl(beg, rr));
						cp[h] = (c < total && tt[h] != t) ? S.sP[tt[h]] : V(0, 0);
					}
#pragma unroll
					for (int h = 0; h < 2; ++h) {
						if (h >= nh) break;
						const int c = base + QG * h + q.sl;
						bool ok = false;
						float d2f = 0;
						if (c < total && tt[h] != t) {
							const float dx = qp.x - cp[h].x, dy = qp.y - cp[h].y;
							d2f = dx * dx + dy * dy;
							if (d2f < r2lo) ok = true;
							else if (d2f <= r2hi) ok = exact_key(qp, cp[h]) < r2d;
						}
						const unsigned m = q_ballot(ok, q);
						if (ok) {
							const int idx = K + __popc(m & q.below);
							if (idx < maxnb) {
								L.ref[idx] = ((uint32_t)g << 28) | (uint32_t)tt[h];
								L.key[idx] = d2f;
							}
						}
						K += __popc(m);
					}
				}
			}
			if (K > maxnb) { *overflow = true; K = maxnb; }
			__syncwarp();
			// one register network (64 entries: a single instantiation keeps
			// the kernel's code small), the shared-memory sort beyond it
			const int len = K - gs;
			const int lmax = q_max(len);
			const float win = lmax <= 64 ? 0x1p-16f : 1e-6f;
			int f0, f1;
			if (lmax <= 64) {
				group_sort_regs<QG, 8>(L, gs, len, q.sl, win, &f0, &f1);
			} else {
				q_sort_smem(S, L, gs, len, lmax, q);
				q_near_ties(L, gs, K, q, win, &f0, &f1);
			}
			q_fix_near_ties(S, L, gs, f0, f1, qp, q, win);
		}
		if (g == 0) K0 = K;
	}
	// PhantomAgent::distSqr of the displaced entries (see gather)
	const int dmax = q_max(K - K0);
	for (int b = 0; b < dmax; b += QG) {
		const int k = K0 + b + q.sl;
		if (k < K) {
			const uint32_t rr = L.ref[k];
			const float2 ph = vadd(S.sP[rr & 0x0FFFFFFFu], group_offset(rr >> 28, W, H));
			L.key[k] = vsq(vsub(p, ph));
		}
	}
	__syncwarp();
	return K;
}

// force_and_contact for an agent's eight lanes, writing the force terms in
// place.  c: the agent's neighbour cost (null: none, or a zero preferred
// velocity); contact_scale 0: no contact forces.  Returns the cost's force
// (agents, then the (0, 0) of the absent obstacles), on all of the agent's
// lanes.
// SF: every neighbour cost of the launch is SocialForces (PowerLaw's code left out)
template <bool SF = false>
__device__ float2 q_force(const DevState& S, const AgentCtx& A, const WarpLists& L, int K, const CostDesc* c,
                          float contact_scale, float W, float H, const QLane& q, float2* contact)
{
	const float rs = c ? c->range * c->range : -1.0f;
	const bool sf = SF || (c && c->kind == K_SOCIALFORCES);
	SfConst SK = {};
	if (c) SK = sf_const(A, *c);
	float2 cacc = V(0, 0);
	const int kmax = q_max(K);
	for (int b0 = 0; b0 < kmax; b0 += QG) {
		const int k = b0 + q.sl;
		bool take = false;
		float2 fc = V(0, 0);
		if (k < K) {
			const uint32_t rr = L.ref[k];
			const int j = (int)(rr & 0x0FFFFFFFu);
			const float2 np = vadd(S.sP[j], group_offset(rr >> 28, W, H));
			const float4 E = S.sE[j];   // (normalised preferred velocity, speed, radius)
			const float nr = E.w;
			const float d2 = L.key[k];
			float2 f = V(0, 0);
			if (d2 <= rs) {
				if (SF || sf) f = sf_force(A, SK, np, E, nr);
				else if constexpr (!SF) f = pl_force(A, *c, np, S.sV[j], nr);
			}
			L.key[k] = f.x;
			L.ref[k] = __float_as_uint(f.y);
			if (contact_scale > 0) {
				// policy.cpp:107-125 (see force_and_contact)
				const float rsum = A.radius + nr;
				if (!(d2 > rsum * rsum * 1.00001f)) {
					const float2 diff = vsub(A.pos, np);
					const float inter = rsum - vmag(diff);
					if (inter > 0) { take = true; fc = vmul(vnorm(diff), contact_scale * inter); }
				}
			}
		}
		// contact terms added in list order
		unsigned m = q_ballot(take, q);
		while (__any_sync(0xffffffffu, m != 0u)) {
			const int src = m ? __ffs(m) - 1 : 0;
			const float fx = q_shfl(fc.x, src), fy = q_shfl(fc.y, src);
			if (m) {
				cacc.x += fx;
				cacc.y += fy;
				m &= m - 1;
			}
		}
	}
	*contact = cacc;
	__syncwarp();
	// the sums in list order: lane 0 the x terms, lane 1 the y terms
	float acc = 0.0f;
	if (c && q.sl < 2) {
		const uint32_t* src = q.sl ? L.ref : reinterpret_cast<const uint32_t*>(L.key);
		int k = 0;
		for (; k + 8 <= K; k += 8) {
			float v[8];
#pragma unroll
			for (int jj = 0; jj < 8; ++jj) v[jj] = __uint_as_float(src[k + jj]);
#pragma unroll
			for (int jj = 0; jj < 8; ++jj) acc += v[jj];
		}
		for (; k < K; ++k) acc += __uint_as_float(src[k]);
	}
	const float2 sum = V(q_shfl(acc, 0), q_shfl(acc, 1));
	__syncwarp();
	return vadd(sum, V(0, 0));
}

constexpr int QPAD = 8;
__host__ __device__ constexpr size_t q_words(int maxnb) { return 2 * (size_t)maxnb + QPAD; }

// One group of four agents (qi: its index in the launch's range) of
// k_force_quad: the gather, the force pass, the agents' records; every 32
// records, the per-agent remainder.
template <bool TAPE, bool SAMP, bool SF>
__device__ __forceinline__ void quad_step(const DevState& S, const QLane& q, const WarpLists& L, float* stash,
                                          int lane, int qi, int& nb, bool& overflow)
{
	const int maxnb = S.maxnb;
	const int t = S.t_begin + qi * QN + q.sg;
	const bool valid = t < S.t_end;
	const int tc = valid ? t : S.t_end - 1;   // in-range loads for a missing fourth agent
	const int slot = S.sSlot[tc];
	const float4 sb = S.sB[tc];
	const float4 prm = S.prm[slot];
	const PolicyDesc& pol = S.pols[S.pol[slot]];
	AgentCtx A;
	A.pos = S.sP[tc]; A.vel = S.sV[tc]; A.pref = V(sb.x, sb.y); A.goal = V(0, 0);
	A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
	const int sc = S.agent_scen[slot];
	const ScenDesc& sd = S.scen[sc];
	const GridParams G = S.grid[sc];
	A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;
	const float W = sd.width, H = sd.height;

	const int K = q_gather(S, G, S.cell_base[sc], sd.world, W, H, L, t, A.pos, pol.range, valid, q, &overflow);
	if (TAPE) {
		const int kmax = q_max(K);
		for (int b = 0; b < kmax; b += QG) {
			const int k = b + q.sl;
			if (k < K) {
				const uint32_t rr = L.ref[k];
				S.tape_list[(size_t)slot * maxnb + k] = (rr & 0xF0000000u) | (uint32_t)S.sSlot[rr & 0x0FFFFFFFu];
			}
		}
		if (valid && q.sl == 0) S.tape_cnt[slot] = K;
		__syncwarp();
	}
	int ci = -1;
	for (int k = 0; k < pol.ncost; ++k)
		if (pol.cost[k].kind != K_GOALREACHING) ci = k;
	const CostDesc* cd = (valid && ci >= 0 && !viszero(A.pref)) ? &pol.cost[ci] : nullptr;
	float2 contact;
	const float2 f = q_force<SF>(S, A, L, K, cd, valid ? pol.contact_scale : 0.0f, W, H, q, &contact);
	if (valid && q.sl == 0) {
		float* rec = stash + (nb + q.sg) * STASH_STRIDE;
		rec[0] = __int_as_float(t);
		if (ci >= 0) { rec[1 + 2 * ci] = f.x; rec[2 + 2 * ci] = f.y; }
		rec[2 * MAX_COSTS + 1] = contact.x;
		rec[2 * MAX_COSTS + 2] = contact.y;
	}
	nb += __popc(__ballot_sync(0xffffffffu, valid && q.sl == 0));
	if (nb > 32 - QN) {
		__syncwarp();
		finish_forces<TAPE, SAMP>(S, stash, nb, lane);
		__syncwarp();
		nb = 0;
	}
}

// WL: compiled for the work-list schedule (schedule 2), which it then
// requires; the other schedules use the variant without it.  SF: every
// neighbour cost of the group is SocialForces.
template <bool TAPE, bool SAMP = false, bool WL = false, bool SF = false>
__global__ void __launch_bounds__(128, 8) k_force_quad(DevState S)
{
	extern __shared__ unsigned char smem[];
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
	QLane q;
	q.sg = lane / QG; q.sl = lane % QG; q.shift = QG * q.sg; q.below = (1u << q.sl) - 1u;
	const int maxnb = S.maxnb;
	// an agent's arrays start QPAD words (8 banks) after the previous agent's
	// and its keys QPAD / 2 words after its references, so that the four
	// agents' lanes, and an agent's two summing lanes, fall in distinct banks
	uint32_t* lists = reinterpret_cast<uint32_t*>(smem) + ((size_t)wib * QN + q.sg) * q_words(maxnb);
	const WarpLists L{ lists, reinterpret_cast<float*>(lists + maxnb + QPAD / 2), nullptr, nullptr };
	float* stash = reinterpret_cast<float*>(smem) + (size_t)(blockDim.x >> 5) * QN * q_words(maxnb) + wib * 32 * STASH_STRIDE;
	bool overflow = false;
	const int nq = (S.t_end - S.t_begin + QN - 1) / QN;
	int nb = 0;
	if constexpr (WL) {
		WorkIter w;
		for (int qi = work_first<32 / QN>(S, w, nq, gw, lane); qi >= 0; qi = work_after<32 / QN>(S, w, qi, lane, nq))
			quad_step<TAPE, SAMP, SF>(S, q, L, stash, lane, qi, nb, overflow);
	} else {
		const int per = (nq + S.total_warps - 1) / S.total_warps;
		const int q0 = S.sched ? gw * per : gw, qstride = S.sched ? 1 : S.total_warps;
		const int qend = S.sched ? min(nq, q0 + per) : nq;
		for (int qi = q0; qi < qend; qi += qstride) quad_step<TAPE, SAMP, SF>(S, q, L, stash, lane, qi, nb, overflow);
	}
	if (nb > 0) {
		__syncwarp();
		finish_forces<TAPE, SAMP>(S, stash, nb, lane);
	}
	work_end<WL>(S, lane);
	if (__any_sync(0xffffffffu, overflow) && lane == 0) atomicOr(S.status, ST_NEIGHBOUR_OVERFLOW);
}

}  // namespace umans
