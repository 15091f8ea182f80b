// neighbour query: warp-cooperative radius search over the cell grid,
// register sort of the nearest neighbours, obstacle lists
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// ------------------------------------------------------------------------
// neighbour query (warp-cooperative)
// ------------------------------------------------------------------------
struct WarpLists {
	uint32_t* ref;   // (displacement group << 28) | cell-sorted index
	float* key;      // sort key, then PhantomAgent::distSqr
	int* nid;        // scratch: per-neighbour x terms of the ordered force sums
	float* aux;      // per-neighbour y terms
};

// (key, id) order; ids are read from the cell-sorted copy when keys tie
__device__ __forceinline__ bool nb_less(const DevState& S, const WarpLists& L, int a, int b)
{
	const float ka = L.key[a], kb = L.key[b];
	if (ka != kb) return ka < kb;
	return S.sId[L.ref[a] & 0x0FFFFFFFu] < S.sId[L.ref[b] & 0x0FFFFFFFu];
}
__device__ __forceinline__ void nb_cmpswap(const DevState& S, const WarpLists& L, int lo, int hi)
{
	if (nb_less(S, L, hi, lo)) {
		float k = L.key[lo]; L.key[lo] = L.key[hi]; L.key[hi] = k;
		uint32_t r = L.ref[lo]; L.ref[lo] = L.ref[hi]; L.ref[hi] = r;
	}
}

// ascending bitonic sort of [s, s+len) by (key, id); the network compares
// only i < j pairs with the min going to i, so the missing elements of the
// power-of-two padding behave as +infinity and are simply skipped.
__device__ void warp_sort(const DevState& S, const WarpLists& L, int s, int len, int lane)
{
	if (len <= 1) return;
	int lp = 0;
	while ((1 << lp) < len) ++lp;
	const int halfP = 1 << (lp - 1);   // pairs per stage
	for (int ls = 1; ls <= lp; ++ls) {
		// first step of block size 2^ls: i against its mirror in the block
		const int lh = ls - 1;
		for (int k = lane; k < halfP; k += 32) {
			const int blk = k >> lh, pos = k & ((1 << lh) - 1);
			const int lo = (blk << ls) + pos, hi = (blk << ls) + (1 << ls) - 1 - pos;
			if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
		}
		__syncwarp();
		// half-cleaners with distance 2^lj
		for (int lj = lh - 1; lj >= 0; --lj) {
			for (int k = lane; k < halfP; k += 32) {
				const int lo = ((k >> lj) << (lj + 1)) | (k & ((1 << lj) - 1)), hi = lo + (1 << lj);
				if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
			}
			__syncwarp();
		}
	}
}

// Sort of [s, s+len), len <= 32 * M (M = 1, 2, 4), in registers: each lane
// holds M packed keys (float key bits with the low PB bits replaced by the
// position in the segment; positive floats order like their bit patterns)
// and a shuffle bitonic network sorts them.  The entries (reference and
// full key) are then permuted through registers.  Keys that agree above the low PB
// bits may come out in either order: the near-tie pass that follows
// (relative window 2^(PB-22), twice the 2^(PB-23) truncation) re-orders
// them with the exact double distance and the id.
template <int M>
__device__ __forceinline__ void warp_sort_regs(const WarpLists& L, int s, int len, int lane)
{
	constexpr int PB = (M == 1) ? 5 : (M == 2) ? 6 : 7;
	constexpr uint32_t PMASK = (1u << PB) - 1u;
	uint32_t u[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * 32 + lane;
		u[m] = (i < len) ? ((__float_as_uint(L.key[s + i]) & ~PMASK) | (uint32_t)i) : 0xffffffffu;
	}
	constexpr int P = 32 * M;
#pragma unroll
	for (int size = 2; size <= P; size <<= 1) {
#pragma unroll
		for (int j = size >> 1; j > 0; j >>= 1) {
#pragma unroll
			for (int m = 0; m < M; ++m) {
				const int i = m * 32 + lane;
				const bool up = (i & size) == 0;
				if (j >= 32) {
					const int mm = m ^ (j >> 5);
					if (mm > m) {
						const uint32_t a = u[m], b = u[mm];
						const bool swap = up ? (a > b) : (a < b);
						if (swap) { u[m] = b; u[mm] = a; }
					}
				} else {
					const uint32_t o = __shfl_xor_sync(0xffffffffu, u[m], j);
					const bool lower = (lane & j) == 0;
					// keep the min in the lower position of an ascending pair
					const bool take_min = (lower == up);
					u[m] = take_min ? min(u[m], o) : max(u[m], o);
				}
			}
		}
	}
	float k[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * 32 + lane;
		const int from = s + (int)(u[m] & PMASK);
		k[m] = (i < len) ? L.key[from] : 0.0f;
		u[m] = (i < len) ? L.ref[from] : 0u;
	}
	__syncwarp();
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * 32 + lane;
		if (i < len) {
			L.ref[s + i] = u[m];
			L.key[s + i] = k[m];
		}
	}
	__syncwarp();
}

__device__ __forceinline__ double exact_key(float2 q, float2 c)
{
	// nanoflann L2_Simple_Adaptor<double>::evalMetric (nanoflann.hpp:423-446)
	const double d0 = __dsub_rn((double)q.x, (double)c.x);
	const double d1 = __dsub_rn((double)q.y, (double)c.y);
	return __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
}

// Float keys order the list except within runs of near-equal keys (relative
// gap <= win: 1e-6 after the exact-key sort, 2^-16 or 2^-15 after the
// packed-key register sorts, whose keys are truncated), which lane 0
// re-sorts in the reference's order.  Float keys carry a relative error below
// 2.5e-7 (one rounding of each difference, square and sum), so two keys more
// than 1e-6 apart order as the exact ones do; closer pairs are compared on the
// reference's double distance, then the id.
// insertion sort of the run [r0, r1] (lane 0) in the reference's order
__device__ void sort_run(const DevState& S, const WarpLists& L, int r0, int r1, float2 q)
{
	for (int x = r0 + 1; x <= r1; ++x) {
		const uint32_t rx = L.ref[x];
		const float kx = L.key[x];
		int y = x - 1;
		while (y >= r0) {
			const uint32_t ry = L.ref[y];
			const float ky = L.key[y];
			bool after;   // entry y belongs after entry x
			if (ky - kx > 1e-6f * ky) after = true;
			else if (kx - ky > 1e-6f * kx) after = false;
			else {
				const double dx = exact_key(q, S.sP[rx & 0x0FFFFFFFu]);
				const double dy = exact_key(q, S.sP[ry & 0x0FFFFFFFu]);
				after = dy > dx || (dy == dx && S.sId[ry & 0x0FFFFFFFu] > S.sId[rx & 0x0FFFFFFFu]);
			}
			if (!after) break;
			L.ref[y + 1] = ry; L.key[y + 1] = ky;
			--y;
		}
		L.ref[y + 1] = rx; L.key[y + 1] = kx;
	}
}

__device__ void fix_near_ties(const DevState& S, const WarpLists& L, int s, int e, float2 q, int lane, float win)
{
	// flags of the adjacent pairs (k, k+1) whose keys are within the window,
	// one bit per pair, 32 pairs per word in the (free) aux list.  Runs are
	// the maximal sequences of flagged pairs; re-sorting a run only permutes
	// keys inside it, so all flags can be taken from the keys as sorted.
	unsigned* words = reinterpret_cast<unsigned*>(L.aux);
	const int npairs = e - 1 - s;
	unsigned any = 0;
	for (int w = 0; 32 * w < npairs; ++w) {
		const int k = s + 32 * w + lane;
		bool close = false;
		if (k + 1 < e) {
			const float a = L.key[k], b = L.key[k + 1];
			close = b - a <= win * b;
		}
		const unsigned m = __ballot_sync(0xffffffffu, close);
		if (lane == 0) words[w] = m;
		any |= m;
	}
	if (!any) return;
	__syncwarp();
	if (lane == 0) {
		const int nw = (npairs + 31) / 32;
		int p = 0;   // next pair to look at
		while (p < npairs) {
			// first flagged pair at or after p
			int w = p >> 5;
			unsigned m = words[w] & (~0u << (p & 31));
			while (!m && ++w < nw) m = words[w];
			if (!m) break;
			const int r0 = 32 * w + __ffs(m) - 1;
			// first unflagged pair after it (or the end)
			int u = r0 >> 5;
			unsigned z = ~words[u] & (~0u << (r0 & 31));
			while (!z && ++u < nw) z = ~words[u];
			const int r1 = z ? min(32 * u + __ffs(z) - 1, npairs) : npairs;
			// pairs r0 .. r1-1 flagged: entries r0 .. r1 form the run
			sort_run(S, L, s + r0, s + r1, q);
			p = r1 + 1;
		}
	}
	__syncwarp();
}

// Gathers the neighbour list of the agent at cell-sorted index t.  Returns
// the list length (clamped to maxnb; *overflow set when clamped).  Entries
// are grouped by displacement in the reference's order (worldToric.cpp:61-79)
// and each group is sorted by the reference's double distance, ties by id.
// On return key[] holds PhantomAgent::distSqr (worldBase.h:73-77).
__device__ int gather(const DevState& S, const GridParams& G, int cb, int world, float W, float H, const WarpLists& L,
                      int t, float2 p, float r, int lane, bool* overflow)
{
	int K = 0, K0 = 0;
	const int maxnb = S.maxnb;
	if (!(r > 0)) return 0;   // dist < r*r never holds for r = 0
	const float r2 = r * r;
	const double r2d = (double)r2;
	const float r2lo = r2 * 0.999999f, r2hi = r2 * 1.000001f;
	const unsigned lt = (1u << lane) - 1u;
	for (int g = 0; g < 5; ++g) {
		float2 disp = V(0, 0);
		if (g > 0) {
			if (world != W_TORIC) break;
			bool active;
			// worldToric.cpp:64-76 compares the float p.x - r with the double
			// -0.5*W; -0.5f*W is that value exactly, so the float compare agrees
			if (g == 1) { active = (p.x - r) < -0.5f * W; disp = V(W, 0); }
			else if (g == 2) { active = (p.x + r) > 0.5f * W; disp = V(-W, 0); }
			else if (g == 3) { active = (p.y - r) < -0.5f * H; disp = V(0, H); }
			else { active = (p.y + r) > 0.5f * H; disp = V(0, -H); }
			if (!active) continue;
		}
		const float2 q = vadd(p, disp);
		const int gs = K;
		const int cx0 = cell_coord((q.x - r - G.x0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.nx);
		const int cx1 = cell_coord((q.x + r - G.x0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.nx);
		const int cy0 = cell_coord((q.y - r - G.y0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.ny);
		const int cy1 = cell_coord((q.y + r - G.y0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.ny);
		// rows of cells covering the query square, ROWS at a time: lane k loads
		// the contiguous sorted range of row k, the rows are concatenated and
		// scanned in full 32-lane chunks
		constexpr int ROWS = 8;
		for (int ry = cy0; ry <= cy1; ry += ROWS) {
			const int nr = min(ROWS, cy1 - ry + 1);
			int rs = 0, len = 0;
			if (lane < nr) {
				const int c0 = cb + (ry + lane) * G.nx;
				rs = S.start[c0 + cx0];
				len = S.start[c0 + cx1 + 1] - rs;
			}
			int incl = len;
			for (int o = 1; o < ROWS; o <<= 1) {
				const int v = __shfl_up_sync(0xffffffffu, incl, o);
				if (lane >= o) incl += v;
			}
			// lane k < ROWS holds row k's start in the concatenation (rows past
			// nr are empty and start at the total)
			const int beg = incl - len;
			const int total = __shfl_sync(0xffffffffu, incl, ROWS - 1);
			// two chunks of 32 candidates per pass: both chunks' positions are
			// loaded before either is tested
			for (int base = 0; base < total; base += 64) {
				const int nh = base + 32 < total ? 2 : 1;
				int tt[2];
				float2 cp[2];
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					if (h >= nh) break;
					const int c = base + 32 * h + lane;
					// the last row starting at or before c (binary search over the
					// ROWS starts, held by lanes 0..ROWS-1)
					int r = 0;
#pragma unroll
					for (int step = ROWS / 2; step > 0; step >>= 1)
						if (__shfl_sync(0xffffffffu, beg, r + step) <= c) r += step;
					tt[h] = __shfl_sync(0xffffffffu, rs, r) + (c - __shfl_sync(0xffffffffu, beg, r));
					cp[h] = (c < total && tt[h] != t) ? S.sP[tt[h]] : V(0, 0);
				}
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					if (h >= nh) break;
					const int c = base + 32 * h + lane;
					bool ok = false;
					float d2f = 0;
					if (c < total && tt[h] != t) {
						const float dx = q.x - cp[h].x, dy = q.y - cp[h].y;
						d2f = dx * dx + dy * dy;
						if (d2f < r2lo) ok = true;
						else if (d2f <= r2hi) ok = exact_key(q, cp[h]) < r2d;
					}
					const unsigned m = __ballot_sync(0xffffffffu, ok);
					if (ok) {
						const int idx = K + __popc(m & lt);
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
		if (g == 0) K0 = K;
		__syncwarp();
		const int len = K - gs;
		if (len <= 32) warp_sort_regs<1>(L, gs, len, lane);
		else if (len <= 64) warp_sort_regs<2>(L, gs, len, lane);
		else if (len <= 128) warp_sort_regs<4>(L, gs, len, lane);
		else warp_sort(S, L, gs, len, lane);
		fix_near_ties(S, L, gs, K, q, lane, len <= 64 ? 0x1p-16f : (len <= 128 ? 0x1p-15f : 1e-6f));
	}
	// PhantomAgent position offset = -displacement; distSqr in float.  For
	// the undisplaced group the sort keys are already that value (same
	// operands, same operations), so only displaced entries are recomputed.
	for (int k = K0 + lane; k < K; k += 32) {
		const uint32_t rr = L.ref[k];
		const float2 ph = vadd(S.sP[rr & 0x0FFFFFFFu], group_offset(rr >> 28, W, H));
		L.key[k] = vsq(vsub(p, ph));
	}
	__syncwarp();
	return K;
}

// The edge-grid query of gather_obstacles for one displacement group: the
// cells covering the query square (with a 1% cell margin); an edge is taken
// in the first of them that its own box covers, so once, and the same
// distance test decides; the group's edges are then put in edge (file)
// order.  Appends to out[K..]; returns the new count.
__device__ __forceinline__ int gather_obstacles_grid(const DevState& S, const ScenDesc& sd, float2 q, float r, int g,
                                                  int lane, uint32_t* out, int K)
{
	const float r2 = r * r;
	const unsigned lt = (1u << lane) - 1u;
	const int gs = K;
	const int qx0 = obs_cell((q.x - r - sd.og_x0) * sd.og_inv - 0.01f, 0.0f, 1.0f, sd.og_nx);
	const int qx1 = obs_cell((q.x + r - sd.og_x0) * sd.og_inv + 0.01f, 0.0f, 1.0f, sd.og_nx);
	const int qy0 = obs_cell((q.y - r - sd.og_y0) * sd.og_inv - 0.01f, 0.0f, 1.0f, sd.og_ny);
	const int qy1 = obs_cell((q.y + r - sd.og_y0) * sd.og_inv + 0.01f, 0.0f, 1.0f, sd.og_ny);
	for (int cy = qy0; cy <= qy1; ++cy) {
		const int row = sd.og_start + cy * sd.og_nx;
		const int i0 = S.og_start[row + qx0], i1 = S.og_start[row + qx1 + 1];
		for (int b0 = i0; b0 < i1; b0 += 32) {
			const int it = b0 + lane;
			bool ok = false;
			int e = 0;
			if (it < i1) {
				const int2 item = S.og_items[it];
				e = item.x;
				const int4 ec = S.og_ecell[e];
				if (item.y == max(ec.x, qx0) && cy == max(ec.y, qy0)) {
					const float4 E = S.edges[e];
					ok = dist2_to_segment(q, V(E.x, E.y), V(E.z, E.w)) <= r2;
				}
			}
			const unsigned m = __ballot_sync(0xffffffffu, ok);
			if (ok) out[K + __popc(m & lt)] = (uint32_t)e;
			K += __popc(m);
		}
	}
	__syncwarp();
	// rank sort of the group's edge indices (distinct)
	const int cnt = K - gs;
	if (cnt <= 32) {
		const uint32_t v = lane < cnt ? out[gs + lane] : 0xffffffffu;
		int rank = 0;
		for (int j = 0; j < cnt; ++j) rank += __shfl_sync(0xffffffffu, v, j) < v;
		__syncwarp();
		if (lane < cnt) out[gs + rank] = ((uint32_t)g << 28) | v;
	} else {
		if (lane == 0) {
			for (int a = gs + 1; a < K; ++a) {
				const uint32_t v = out[a];
				int b = a - 1;
				while (b >= gs && out[b] > v) { out[b + 1] = out[b]; --b; }
				out[b + 1] = v;
			}
			for (int a = gs; a < K; ++a) out[a] |= (uint32_t)g << 28;
		}
	}
	__syncwarp();
	return K;
}

// Obstacle edges within range of the agent (worldBase.cpp:62-77), per
// displacement group as the agents (worldToric.cpp:32-79): edges in file
// order, each group's appended after the previous one.  Returns the count.
__device__ int gather_obstacles(const DevState& S, const ScenDesc& sd, float2 p, float r, int lane, uint32_t* out)
{
	int K = 0;
	const float r2 = r * r;
	const unsigned lt = (1u << lane) - 1u;
	for (int g = 0; g < 5; ++g) {
		float2 disp = V(0, 0);
		if (g > 0) {
			if (sd.world != W_TORIC) break;
			bool active;
			if (g == 1) { active = (p.x - r) < -0.5f * sd.width; disp = V(sd.width, 0); }
			else if (g == 2) { active = (p.x + r) > 0.5f * sd.width; disp = V(-sd.width, 0); }
			else if (g == 3) { active = (p.y - r) < -0.5f * sd.height; disp = V(0, sd.height); }
			else { active = (p.y + r) > 0.5f * sd.height; disp = V(0, -sd.height); }
			if (!active) continue;
		}
		const float2 q = vadd(p, disp);
		if (sd.og_nx == 0) {
			for (int b0 = 0; b0 < sd.nedges; b0 += 32) {
				const int k = b0 + lane;
				bool ok = false;
				if (k < sd.nedges) {
					const float4 E = S.edges[sd.edge_off + k];
					ok = dist2_to_segment(q, V(E.x, E.y), V(E.z, E.w)) <= r2;
				}
				const unsigned m = __ballot_sync(0xffffffffu, ok);
				if (ok) out[K + __popc(m & lt)] = ((uint32_t)g << 28) | (uint32_t)(sd.edge_off + k);
				K += __popc(m);
			}
			continue;
		}
		K = gather_obstacles_grid(S, sd, q, r, g, lane, out, K);
		__syncwarp();
	}
	__syncwarp();
	return K;
}

}  // namespace umans
