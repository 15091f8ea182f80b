/* CPU restatement of the UMANS per-step agent update -- TEST INFRASTRUCTURE.
 *
 * This file is the oracle: a plain-C restatement of WorldBase::DoStep
 * (src/Engine/core/worldBase.cpp:79-128) and everything it calls on the hot
 * path.  Tests compare the CUDA engine with it; bench.py times it as the CPU
 * baseline.  It is never linked into the product.
 *
 * Arithmetic follows the reference operation by operation: float where the
 * reference computes in float (Vector2D is float, src/Engine/tools/vector2D.h),
 * double where the reference promotes (acos in angle(), pow(x,2), the
 * rotation in rotateCounterClockwise, getLineIntersection, the kd-tree
 * distance).  Build with -ffp-contract=off so that no a*b+c is fused.
 *
 * Neighbour lists: the reference's nanoflann radius search returns the set
 * {j != i : (double)dx^2 + (double)dy^2 < (double)(r*r)} sorted by that
 * double distance (std::sort, ties in tree order).  Here the same set is
 * found with a uniform grid and sorted by (distance, id); the two orders
 * agree whenever distances differ.
 */
#include "umans_port.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define MAXF FLT_MAX
static const double REF_PI = 3.1415926535897; /* vector2D.h:27 */

/* ------------------------------------------------------------------ */
/* Vector2D (src/Engine/tools/vector2D.h)                              */
/* ------------------------------------------------------------------ */
typedef struct { float x, y; } v2;

static inline v2 V(float x, float y) { v2 r = { x, y }; return r; }
static inline v2 vadd(v2 a, v2 b) { return V(a.x + b.x, a.y + b.y); }
static inline v2 vsub(v2 a, v2 b) { return V(a.x - b.x, a.y - b.y); }
/* operator*(float, Vector2D) and operator*(Vector2D, float): vector2D.h:120-128 */
static inline v2 vmul(v2 a, float s) { return V(a.x * s, a.y * s); }
/* operator/(Vector2D, float) multiplies by the reciprocal: vector2D.h:132-135 */
static inline v2 vdiv(v2 a, float s) { float r = 1.0f / s; return V(a.x * r, a.y * r); }
static inline float vdot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline float vsq(v2 a) { return a.x * a.x + a.y * a.y; }
static inline float vmag(v2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
static inline int viszero(v2 a) { return a.x == 0 && a.y == 0; }
/* normalize(): vector2D.h:41-49 (true division by the magnitude) */
static inline v2 vnorm(v2 a)
{
	float m = vmag(a);
	if (m > 0) { a.x /= m; a.y /= m; }
	return a;
}
/* clampVector: vector2D.h:241-247 */
static inline v2 vclamp(v2 v, float maxLength)
{
	float m = vmag(v);
	if (m <= maxLength) return v;
	return vmul(vnorm(v), maxLength);
}
/* rotateCounterClockwise: vector2D.h:166-170; cos/sin of a float call cosf/sinf */
static inline v2 vrot(v2 v, float radians)
{
	const double c = (double)cosf(radians), s = (double)sinf(radians);
	return V((float)(c * v.x - s * v.y), (float)(s * v.x + c * v.y));
}
/* angle: vector2D.h:172-186 (lengths: float product promoted to double) */
static inline float vangle(v2 a, v2 b)
{
	const double lengths = (double)(vmag(a) * vmag(b));
	if (lengths == 0) return 0.0f;
	const double frac = (double)vdot(a, b) / lengths;
	if (frac < -1 || frac > 1) return 0.0f;
	return (float)acos(frac);
}
/* cosAngle: vector2D.h:188-195 */
static inline float vcosangle(v2 a, v2 b)
{
	const double lengths = (double)(vmag(a) * vmag(b));
	if (lengths == 0) return 0.0f;
	return (float)((double)vdot(a, b) / lengths);
}
static inline int vclockwise(v2 a, v2 b) { float c = a.x * b.y - a.y * b.x; return c < 0; }
/* counterClockwiseAngle: vector2D.h:209-215 */
static inline float vccwangle(v2 a, v2 b)
{
	float ang = vangle(a, b);
	if (vclockwise(a, b)) return -ang;
	return ang;
}
/* getLineIntersection: vector2D.h:249-272 (double) */
static inline int line_intersection(v2 a, v2 b, v2 c, v2 d, v2* res)
{
	double a1 = b.y - a.y, b1 = a.x - b.x;
	double c1 = a1 * a.x + b1 * a.y;
	double a2 = d.y - c.y, b2 = c.x - d.x;
	double c2 = a2 * c.x + b2 * c.y;
	double det = a1 * b2 - a2 * b1;
	if (fabs(det) < 0.00001) return 0;
	res->x = (float)((b2 * c1 - b1 * c2) / det);
	res->y = (float)((a1 * c2 - a2 * c1) / det);
	return 1;
}
static inline float fminr(float a, float b) { return (b < a) ? b : a; } /* std::min */
static inline float fmaxr(float a, float b) { return (a < b) ? b : a; } /* std::max */

/* ------------------------------------------------------------------ */
/* world state                                                         */
/* ------------------------------------------------------------------ */
typedef struct {
	int j;          /* slot of the neighbour */
	v2 pos;         /* neighbour position + offset (PhantomAgent::position) */
	float d2;       /* PhantomAgent::distSqr (float) */
	double key;     /* kd-tree double distance to the (displaced) query */
} nbr;

typedef struct { nbr* v; int n, cap; } nbrlist;
typedef struct { v2 a, b; } seg;
typedef struct { seg* v; int n, cap; } seglist;

struct up_world {
	int n, type;
	float width, height, dt;
	double time;
	up_policy* pol;
	int npol;
	long long* id;
	v2 *pos, *vel, *goal, *pref, *next, *vwf, *view, *contact;
	float *radius, *prefspeed, *maxspeed, *maxacc;
	int* policy;
	uint32_t* rng;
	nbrlist* nb;
	/* obstacle edges (Polygon2D edges in file order) and each agent's list */
	seg* edges;
	int ne;
	seglist* ob;
	/* grid */
	int *cell_start, *cell_items, gnx, gny, gcells_cap;
	float gx0, gy0, gcs;
	/* dynamic population (worldBase.cpp:79-86, 124-127, 161-235): the arrays
	 * above hold the current agent list in its order, with room for every
	 * agent; agents with a start time wait in `pend` (file order, stably
	 * sorted by start time) */
	unsigned char* rmg;      /* remove at goal, per list slot (or NULL) */
	int cap;
	struct up_pending* pend;
	int npend, next_pend;
};

struct up_pending {
	long long id;
	v2 pos, goal;
	float radius, prefspeed, maxspeed, maxacc, start;
	int policy;
	unsigned char rmg;
};

/* ------------------------------------------------------------------ */
/* RNG: std::default_random_engine = minstd_rand0 (agent.cpp:38,131-135)*/
/* ------------------------------------------------------------------ */
static inline uint32_t minstd_seed(uint64_t s)
{
	uint32_t x = (uint32_t)(s % 2147483647u);
	return x == 0 ? 1u : x;
}
static inline float rng_uniform(uint32_t* st, float a, float b)
{
	/* generate_canonical<float,24> with one draw (libstdc++ random.tcc) */
	*st = (uint32_t)(((uint64_t)(*st) * 16807u) % 2147483647u);
	float sum = (float)(unsigned long)(*st - 1u);
	float ret = sum / 2147483648.0f;
	if (ret >= 1.0f) ret = nextafterf(1.0f, 0.0f);
	return ret * (b - a) + a;
}

/* ------------------------------------------------------------------ */
/* neighbour search (AgentKDTree.cpp:35-59, worldInfinite.cpp:31-52,   */
/* worldToric.cpp:32-79, worldBase.h:56-77)                            */
/* ------------------------------------------------------------------ */
static float policy_range(const up_policy* p)   /* policy.cpp:34-41 */
{
	float r = 0;
	for (int c = 0; c < p->ncost; ++c) r = fmaxr(r, p->cost[c].range);
	return r;
}

static void grid_build(up_world* w)
{
	float maxr = 0;
	for (int k = 0; k < w->npol; ++k) maxr = fmaxr(maxr, policy_range(&w->pol[k]));
	float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
	for (int i = 0; i < w->n; ++i) {
		x0 = fminf(x0, w->pos[i].x); x1 = fmaxf(x1, w->pos[i].x);
		y0 = fminf(y0, w->pos[i].y); y1 = fmaxf(y1, w->pos[i].y);
	}
	if (w->n == 0) { x0 = y0 = 0; x1 = y1 = 1; }
	float cs = maxr > 0.05f ? maxr : 0.05f;
	double ex = (double)x1 - x0, ey = (double)y1 - y0;
	while ((ex / cs + 1) * (ey / cs + 1) > 8.0 * w->n + 1024) cs *= 2;
	int nx = (int)(ex / cs) + 1, ny = (int)(ey / cs) + 1;
	int cells = nx * ny;
	if (cells + 1 > w->gcells_cap) {
		free(w->cell_start);
		w->gcells_cap = cells + 1;
		w->cell_start = (int*)malloc(sizeof(int) * (size_t)w->gcells_cap);
	}
	w->gnx = nx; w->gny = ny; w->gx0 = x0; w->gy0 = y0; w->gcs = cs;
	memset(w->cell_start, 0, sizeof(int) * (size_t)(cells + 1));
	int* cell = (int*)malloc(sizeof(int) * (size_t)(w->n + 1));
	for (int i = 0; i < w->n; ++i) {
		int cx = (int)((w->pos[i].x - x0) / cs), cy = (int)((w->pos[i].y - y0) / cs);
		if (cx >= nx) cx = nx - 1;
		if (cy >= ny) cy = ny - 1;
		cell[i] = cy * nx + cx;
		w->cell_start[cell[i] + 1]++;
	}
	for (int c = 0; c < cells; ++c) w->cell_start[c + 1] += w->cell_start[c];
	int* fill = (int*)malloc(sizeof(int) * (size_t)(cells + 1));
	memcpy(fill, w->cell_start, sizeof(int) * (size_t)(cells + 1));
	free(w->cell_items);
	w->cell_items = (int*)malloc(sizeof(int) * (size_t)(w->n + 1));
	for (int i = 0; i < w->n; ++i) w->cell_items[fill[cell[i]]++] = i;
	free(fill);
	free(cell);
}

static void nb_push(nbrlist* L, nbr e)
{
	if (L->n == L->cap) {
		L->cap = L->cap ? L->cap * 2 : 32;
		L->v = (nbr*)realloc(L->v, sizeof(nbr) * (size_t)L->cap);
	}
	L->v[L->n++] = e;
}

static int nbr_cmp(const void* a, const void* b, void* ctx)
{
	const nbr* x = (const nbr*)a; const nbr* y = (const nbr*)b;
	const long long* id = (const long long*)ctx;
	if (x->key < y->key) return -1;
	if (x->key > y->key) return 1;
	return (id[x->j] < id[y->j]) ? -1 : (id[x->j] > id[y->j]);
}

/* insertion sort on (key, id); lists are short */
static void nb_sort(nbr* v, int n, const long long* id)
{
	for (int a = 1; a < n; ++a) {
		nbr e = v[a];
		int b = a - 1;
		while (b >= 0 && nbr_cmp(&v[b], &e, (void*)id) > 0) { v[b + 1] = v[b]; --b; }
		v[b + 1] = e;
	}
}

/* one kd-style radius query at q (already displaced), appended to L with
 * PhantomAgent offset `off` relative to the undisplaced query `q0` */
static void query_group(const up_world* w, int self, v2 q0, v2 q, float r, v2 off, nbrlist* L)
{
	const double r2 = (double)(r * r);
	int start = L->n;
	const float cs = w->gcs;
	int cx0 = (int)floor(((double)q.x - r - w->gx0) / cs), cx1 = (int)floor(((double)q.x + r - w->gx0) / cs);
	int cy0 = (int)floor(((double)q.y - r - w->gy0) / cs), cy1 = (int)floor(((double)q.y + r - w->gy0) / cs);
	if (cx0 < 0) cx0 = 0;
	if (cy0 < 0) cy0 = 0;
	if (cx1 >= w->gnx) cx1 = w->gnx - 1;
	if (cy1 >= w->gny) cy1 = w->gny - 1;
	for (int cy = cy0; cy <= cy1; ++cy)
		for (int cx = cx0; cx <= cx1; ++cx) {
			int c = cy * w->gnx + cx;
			for (int t = w->cell_start[c]; t < w->cell_start[c + 1]; ++t) {
				int j = w->cell_items[t];
				if (j == self) continue;
				double d0 = (double)q.x - (double)w->pos[j].x;
				double d1 = (double)q.y - (double)w->pos[j].y;
				double dist = d0 * d0;
				dist += d1 * d1;
				if (dist < r2) {
					nbr e;
					e.j = j;
					e.pos = vadd(w->pos[j], off);
					e.d2 = vsq(vsub(q0, e.pos));
					e.key = dist;
					nb_push(L, e);
				}
			}
		}
	nb_sort(L->v + start, L->n - start, w->id);
}

/* nearestPointOnLine(pt, la, lb, onSegment = true): vector2D.h:274-296 */
static inline v2 nearest_on_segment(v2 pt, v2 la, v2 lb)
{
	if (la.x == lb.x && la.y == lb.y) return la;
	const v2 line = vsub(la, lb);
	float k = vdot(vsub(pt, lb), line) / vsq(line);
	if (k > 1) k = 1;
	else if (k < 0) k = 0;
	return vadd(vmul(la, k), vmul(lb, 1 - k));
}
/* distanceToLineSquared(pt, la, lb, true): vector2D.h:303-306 */
static inline float dist2_to_segment(v2 pt, v2 la, v2 lb) { return vsq(vsub(pt, nearest_on_segment(pt, la, lb))); }

static void seg_push(seglist* L, seg e)
{
	if (L->n == L->cap) {
		L->cap = L->cap ? 2 * L->cap : 16;
		L->v = (seg*)realloc(L->v, sizeof(seg) * (size_t)L->cap);
	}
	L->v[L->n++] = e;
}

/* computeNeighboringObstacles_Flat (worldBase.cpp:62-77) at the displaced
 * query point q, edges shifted by -displacement (worldToric.cpp:50-58) */
static void query_obstacles(const up_world* w, v2 q, float r, v2 disp, int displaced, seglist* L)
{
	const float r2 = r * r;
	for (int k = 0; k < w->ne; ++k) {
		const seg e = w->edges[k];
		if (dist2_to_segment(q, e.a, e.b) <= r2) {
			seg o = e;
			if (displaced) { o.a = vsub(e.a, disp); o.b = vsub(e.b, disp); }
			seg_push(L, o);
		}
	}
}

static void compute_neighbors(up_world* w, int i)
{
	nbrlist* L = &w->nb[i];
	seglist* O = &w->ob[i];
	L->n = 0;
	O->n = 0;
	const float r = policy_range(&w->pol[w->policy[i]]);
	const v2 p = w->pos[i];
	query_group(w, i, p, p, r, V(0, 0), L);
	query_obstacles(w, p, r, V(0, 0), 0, O);
	if (w->type == UP_TORIC) {
		const float W = w->width, H = w->height;
		/* worldToric.cpp:61-79: four axis displacements, no diagonals */
		if (p.x - r < -0.5 * W) {
			query_group(w, i, p, vadd(p, V(W, 0)), r, V(-W, -0.0f), L);
			query_obstacles(w, vadd(p, V(W, 0)), r, V(W, 0), 1, O);
		}
		if (p.x + r > 0.5 * W) {
			query_group(w, i, p, vadd(p, V(-W, 0)), r, V(W, -0.0f), L);
			query_obstacles(w, vadd(p, V(-W, 0)), r, V(-W, 0), 1, O);
		}
		if (p.y - r < -0.5 * H) {
			query_group(w, i, p, vadd(p, V(0, H)), r, V(-0.0f, -H), L);
			query_obstacles(w, vadd(p, V(0, H)), r, V(0, H), 1, O);
		}
		if (p.y + r > 0.5 * H) {
			query_group(w, i, p, vadd(p, V(0, -H)), r, V(-0.0f, H), L);
			query_obstacles(w, vadd(p, V(0, -H)), r, V(0, -H), 1, O);
		}
	}
}

/* ------------------------------------------------------------------ */
/* shared cost helpers (costFunction.cpp:173-268, 354-380)             */
/* ------------------------------------------------------------------ */
static inline int solve_quadratic(float a, float b, float c, float* x1, float* x2)
{
	const float D = b * b - 4 * a * c;
	if (D < 0) return 0;
	if (D == 0) { *x1 = -b / 2 * a; return 1; }  /* sic: costFunction.cpp:180 */
	const float m = -b / (2 * a);
	const float s = sqrtf(D) / (2 * a);
	*x1 = m + s;
	*x2 = m - s;
	return 2;
}

static inline float ttc_pair(v2 p1, v2 v1, float r1, v2 p2, v2 v2_, float r2)
{
	const v2 P = vsub(p1, p2);
	const float R = r1 + r2, RR = R * R;
	if (vsq(P) <= RR) return 0;
	const v2 Vd = vsub(v1, v2_);
	const float a = vdot(Vd, Vd), b = 2 * vdot(P, Vd), c = vdot(P, P) - RR;
	float t1 = MAXF, t2 = MAXF;
	solve_quadratic(a, b, c, &t1, &t2);
	if (t1 < 0) t1 = MAXF;
	if (t2 < 0) t2 = MAXF;
	return fminr(t1, t2);
}

/* ComputeTimeToCollision_LineSegmentInterior: costFunction.cpp:293-325 */
static float ttc_segment_interior(v2 p, v2 v, float r, v2 a, v2 b)
{
	if (dist2_to_segment(p, a, b) <= r * r) return 0;
	v2 X;
	if (!line_intersection(p, vadd(p, v), a, b, &X)) return MAXF;
	if (vdot(v, vsub(X, p)) < 0) return MAXF;
	const v2 line = vsub(a, b);
	const float k = vdot(vsub(X, b), line) / vsq(line);
	if (!(k >= 0 && k <= 1)) return MAXF;
	const float speed = vmag(v);
	const float t = vmag(vsub(X, p)) / speed;
	const float ang = vangle(v, vsub(b, a));
	const float sub = r / sinf(ang);
	const float tsub = sub / speed;
	return fmaxr(0.0f, t - tsub);
}

/* ComputeTimeToCollision_LineSegment: costFunction.cpp:270-291 */
static float ttc_segment(v2 p, v2 v, float r, v2 a, v2 b)
{
	const float t1 = ttc_pair(p, v, r, a, V(0, 0), 0);
	if (t1 == 0) return 0;
	if (a.x == b.x && a.y == b.y) return t1;
	const float t2 = ttc_pair(p, v, r, b, V(0, 0), 0);
	if (t2 == 0) return 0;
	const float ti = ttc_segment_interior(p, v, r, a, b);
	return fminr(fminr(t1, t2), ti);
}

typedef struct {
	const up_world* w;
	int i;
	const nbrlist* L;
	const seglist* O;
	v2 pos, vel, pref, goal;
	float radius, prefspeed, maxspeed, maxacc, dt, relax;
} actx;

static inline float ttc_first(const actx* A, v2 pos, v2 vel, float radius, float maxDist, int ignoreCurrent)
{
	float minT = MAXF;
	const float md2 = maxDist * maxDist;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 > md2) continue;
		float t = ttc_pair(pos, vel, radius, e->pos, A->w->vel[e->j], A->w->radius[e->j]);
		if (ignoreCurrent && t == 0) continue;
		if (t < minT) minT = t;
	}
	/* neighbouring obstacles: costFunction.cpp:251-265 */
	for (int k = 0; k < A->O->n; ++k) {
		const seg e = A->O->v[k];
		if (dist2_to_segment(pos, e.a, e.b) > md2) continue;
		float t = ttc_segment(pos, vel, radius, e.a, e.b);
		if (ignoreCurrent && t == 0) continue;
		if (t < minT) minT = t;
	}
	return minT;
}

static inline void ttca_dca(v2 p1, v2 v1, float r1, v2 p2, v2 v2_, float r2, float* ttca_out, float* dca_out)
{
	const v2 dpc = vsub(p2, p1), dvc = vsub(v2_, v1);
	float dpMag = vmag(dpc);
	const v2 dp = vmul(vdiv(dpc, dpMag), dpMag - r1 - r2);
	v2 nrm = V(-dpc.y, dpc.x);
	const v2 dv = vadd(dvc, vmul(nrm, vdot(nrm, dvc)));
	float ttca = (vsq(dv) == 0 ? 0 : -vdot(dp, dv) / vsq(dv));
	if (ttca < 0) ttca = 0;
	float dca = vmag(vadd(dp, vmul(dv, ttca)));
	if (dca < 0) dca = 0;
	*ttca_out = ttca;
	*dca_out = dca;
}

/* RotateGradientToEuclideanCoordinates: costFunction.cpp:30-34 */
static inline v2 rotate_gradient(float gth, float gs, v2 dir, float speed)
{
	v2 w = vadd(vmul(V(sinf(gth), 1 - cosf(gth)), speed), V(0, gs));
	/* Matrix(Vector2D(dir.y,-dir.x), dir) * w  (Matrix.h) */
	return V(dir.y * w.x + dir.x * w.y, -dir.x * w.x + dir.y * w.y);
}

/* ------------------------------------------------------------------ */
/* force-based costs (ForceBasedFunction.cpp, ObjectInteractionForces.cpp) */
/* ------------------------------------------------------------------ */
static v2 sf_force(const actx* A, const up_cost* c, const nbr* e)
{   /* SocialForcesAvoidance.cpp:26-110 */
	const up_world* w = A->w;
	const float dtp = c->p[0], V0 = c->p[1], sigma = c->p[2];
	const v2 R = vsub(A->pos, e->pos);
	float magR = vmag(R);
	if (magR <= A->radius + w->radius[e->j]) return V(0, 0);
	float vb = vmag(w->vel[e->j]);
	const v2 Eb = vnorm(w->pref[e->j]);
	const v2 Vv = vmul(Eb, vb * dtp);
	float magV = vmag(Vv);
	const v2 R2 = vsub(R, Vv);
	float magR2 = vmag(R2);
	double s = (double)(magR + magR2), t = (double)(vb * dtp);
	float bSquared2 = (float)(s * s - t * t);
	if (bSquared2 <= 0) return V(0, 0);
	float b = 0.5f * sqrtf(bSquared2);
	if (b < 0.001f) return V(0, 0);
	const float d_magR2 = 1 / (2 * magR2) * (2 * magR - 2 * magV * vcosangle(R, Vv));
	const float d_bSquared2 = 2 * (magR + magR2) * (1 + d_magR2);
	const float d_b = (1 / (8 * b)) * d_bSquared2;
	const float d_V = -V0 / sigma * expf(-b / sigma) * d_b;
	const v2 F = vmul(V(-R.x, -R.y), d_V);
	const float viewHalf = (float)(100.0 * REF_PI / 180.0);
	float scale = (vangle(A->vel, V(-R.x, -R.y)) < viewHalf ? 1 : 0.5f);
	return vmul(F, scale);
}

static v2 pl_force(const actx* A, const up_cost* c, const nbr* e)
{   /* PowerLaw.cpp:28-66 */
	const up_world* w = A->w;
	const float k = c->p[0], tau0 = c->p[1];
	float R = w->radius[e->j] + A->radius;
	const v2 x = vsub(A->pos, e->pos);
	const v2 v = vsub(A->vel, w->vel[e->j]);
	float a = vdot(v, v), b = -vdot(x, v), cc = vdot(x, x) - R * R;
	if (cc <= 0) return V(0, 0);
	float d = b * b - a * cc;
	if (d <= 0) return V(0, 0);
	float sqrtD = sqrtf(d);
	float tau = (b - sqrtD) / a;
	if (tau < 0.001f) return V(0, 0);
	if (tau > tau0) return V(0, 0);
	float comp1 = -k * expf(-tau / tau0) * (2 / tau + 1 / tau0) / (a * tau * tau);
	const v2 comp2 = vsub(v, vdiv(vadd(vmul(x, a), vmul(v, b)), sqrtD));
	return vmul(comp2, comp1);
}

static v2 compute_force(const actx* A, const up_cost* c)
{
	if (c->kind == UP_GOALREACHING)   /* GoalReachingForce.cpp:26-29 */
		return vdiv(vsub(A->pref, A->vel), fmaxr(A->relax, A->dt));
	/* ObjectInteractionForces::ComputeForce: ObjectInteractionForces.cpp:26-48 */
	const float rs = c->range * c->range;
	v2 F = V(0, 0);
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 <= rs) {
			v2 f = (c->kind == UP_SOCIALFORCES) ? sf_force(A, c, e) : pl_force(A, c, e);
			F.x += f.x; F.y += f.y;
		}
	}
	v2 O = V(0, 0);
	for (int k = 0; k < A->O->n; ++k) {
		const seg e = A->O->v[k];
		if (dist2_to_segment(A->pos, e.a, e.b) <= rs) {
			v2 f = V(0, 0);   /* PowerLaw: no obstacle force (PowerLaw.cpp:68-72) */
			if (c->kind == UP_SOCIALFORCES) {
				/* SocialForcesAvoidance::ComputeObstacleInteractionForce: .cpp:112-140 */
				const v2 diff = vsub(A->pos, nearest_on_segment(A->pos, e.a, e.b));
				const float dist = vmag(diff);
				if (!(dist < 0.001f)) {
					const float U0 = c->p[3], R = c->p[4];
					const float dU = -U0 / R * expf(-dist / R);
					f = vmul(V(-diff.x, -diff.y), dU);
				}
			}
			O.x += f.x; O.y += f.y;
		}
	}
	return vadd(F, O);
}

static v2 target_velocity(const actx* A, const up_cost* c)
{   /* ForceBasedFunction.cpp:48-52 */
	return vadd(A->vel, vmul(vdiv(compute_force(A, c), c->p[5]), A->dt));
}

/* ------------------------------------------------------------------ */
/* ORCA (CostFunctions/ORCA.cpp, 3rd-party/ORCA/ORCASolver.cpp)        */
/* ------------------------------------------------------------------ */
typedef struct { v2 point, dir; } oline;
static const float ORCA_EPS = 0.00001f;
static inline float det2(v2 a, v2 b) { return a.x * b.y - a.y * b.x; }

static int lp1(const oline* L, int lineNo, float radius, v2 opt, int dirOpt, v2* res)
{
	const float dp = vdot(L[lineNo].point, L[lineNo].dir);
	const float disc = dp * dp + radius * radius - vsq(L[lineNo].point);
	if (disc < 0.0f) return 0;
	const float sd = sqrtf(disc);
	float tl = -dp - sd, tr = -dp + sd;
	for (int i = 0; i < lineNo; ++i) {
		const float den = det2(L[lineNo].dir, L[i].dir);
		const float num = det2(L[i].dir, vsub(L[lineNo].point, L[i].point));
		if (fabsf(den) <= ORCA_EPS) {
			if (num < 0.0f) return 0;
			continue;
		}
		const float t = num / den;
		if (den >= 0.0f) tr = fminr(tr, t);
		else tl = fmaxr(tl, t);
		if (tl > tr) return 0;
	}
	if (dirOpt) {
		if (vdot(opt, L[lineNo].dir) > 0.0f) *res = vadd(L[lineNo].point, vmul(L[lineNo].dir, tr));
		else *res = vadd(L[lineNo].point, vmul(L[lineNo].dir, tl));
	} else {
		const float t = vdot(L[lineNo].dir, vsub(opt, L[lineNo].point));
		if (t < tl) *res = vadd(L[lineNo].point, vmul(L[lineNo].dir, tl));
		else if (t > tr) *res = vadd(L[lineNo].point, vmul(L[lineNo].dir, tr));
		else *res = vadd(L[lineNo].point, vmul(L[lineNo].dir, t));
	}
	return 1;
}

static int lp2(const oline* L, int n, float radius, v2 opt, int dirOpt, v2* res)
{
	if (dirOpt) *res = vmul(opt, radius);
	else if (vsq(opt) > radius * radius) *res = vmul(vnorm(opt), radius);
	else *res = opt;
	for (int i = 0; i < n; ++i) {
		if (det2(L[i].dir, vsub(L[i].point, *res)) > 0.0f) {
			const v2 tmp = *res;
			if (!lp1(L, i, radius, opt, dirOpt, res)) { *res = tmp; return i; }
		}
	}
	return n;
}

static void lp3(const oline* L, int n, int begin, float radius, v2* res, oline* proj)
{
	float distance = 0.0f;
	for (int i = begin; i < n; ++i) {
		if (det2(L[i].dir, vsub(L[i].point, *res)) > distance) {
			int np = 0;
			for (int j = 0; j < i; ++j) {
				oline ln;
				float determinant = det2(L[i].dir, L[j].dir);
				if (fabsf(determinant) <= ORCA_EPS) {
					if (vdot(L[i].dir, L[j].dir) > 0.0f) continue;
					ln.point = vmul(vadd(L[i].point, L[j].point), 0.5f);
				} else {
					ln.point = vadd(L[i].point, vmul(L[i].dir, det2(L[j].dir, vsub(L[i].point, L[j].point)) / determinant));
				}
				ln.dir = vnorm(vsub(L[j].dir, L[i].dir));
				proj[np++] = ln;
			}
			const v2 tmp = *res;
			if (lp2(proj, np, radius, V(-L[i].dir.y, L[i].dir.x), 1, res) < np) *res = tmp;
			distance = det2(L[i].dir, vsub(L[i].point, *res));
		}
	}
}

typedef struct { v2 velocity; oline* lines; int nlines; } orca_sol;

static void orca_solve(const actx* A, const up_cost* c, orca_sol* S)
{   /* Solver::solveOrcaProgram + createAgentOrcaLines: ORCASolver.cpp:61-171 */
	const float tH = c->p[0];
	const float maxDistSq = c->range * c->range;
	const float rad = A->radius;
	S->lines = (oline*)malloc(sizeof(oline) * (size_t)(A->L->n + 1));
	S->nlines = 0;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 > maxDistSq) continue;
		const v2 relPos = vsub(e->pos, A->pos);
		const v2 relVel = vsub(A->vel, A->w->vel[e->j]);
		const float distSq = vsq(relPos);
		const float cR = rad + A->w->radius[e->j];
		const float cRSq = cR * cR;
		oline line;
		v2 u;
		if (distSq > cRSq) {
			const v2 w = vsub(relVel, vdiv(relPos, tH));
			const float wLenSq = vsq(w);
			const float dp1 = vdot(w, relPos);
			if (dp1 < 0.0f && dp1 * dp1 > cRSq * wLenSq) {
				const float wLen = sqrtf(wLenSq);
				const v2 unitW = vdiv(w, wLen);
				line.dir = V(unitW.y, -unitW.x);
				u = vmul(unitW, cR / tH - wLen);
			} else {
				const float leg = sqrtf(distSq - cRSq);
				if (det2(relPos, w) > 0.0f)
					line.dir = vdiv(V(relPos.x * leg - relPos.y * cR, relPos.x * cR + relPos.y * leg), distSq);
				else
					line.dir = vdiv(vmul(V(relPos.x * leg + relPos.y * cR, -relPos.x * cR + relPos.y * leg), -1), distSq);
				const float dp2 = vdot(relVel, line.dir);
				u = vsub(vmul(line.dir, dp2), relVel);
			}
		} else {
			const v2 w = vsub(relVel, vdiv(relPos, A->dt));
			const float wLen = vsq(w);   /* sic: ORCASolver.cpp:161 */
			const v2 unitW = vdiv(w, wLen);
			line.dir = V(unitW.y, -unitW.x);
			u = vmul(unitW, cR / A->dt - wLen);
		}
		line.point = vadd(A->vel, vmul(u, 0.5f));
		S->lines[S->nlines++] = line;
	}
	int fail = lp2(S->lines, S->nlines, A->maxspeed, A->pref, 0, &S->velocity);
	if (fail < S->nlines) {
		oline* proj = (oline*)malloc(sizeof(oline) * (size_t)(S->nlines + 1));
		lp3(S->lines, S->nlines, fail, A->maxspeed, &S->velocity, proj);
		free(proj);
	}
}

/* ------------------------------------------------------------------ */
/* per-sample costs                                                    */
/* ------------------------------------------------------------------ */
typedef struct {
	/* per-agent invariants computed once per cost function per step */
	v2 target;          /* force-based: target velocity */
	float ttc_pref;     /* Karamouzas: TTC at the preferred velocity */
	orca_sol orca;      /* ORCA: lines and solution */
	int has_orca;
} cprep;

static float cost_eval(const actx* A, const up_cost* c, cprep* P, v2 v);

static float karamouzas_maxdev(float ttc)
{   /* Karamouzas.cpp:115-123; tc_max stays at the default 8 (Karamouzas.h:58) */
	const float tc_min = 2.5f, tc_mid = 6, tc_max = 8;
	const float d_min = 0.05f, d_mid = (float)(REF_PI / 6.0f), d_max = (float)(REF_PI / 2.0f);
	if (ttc <= 0 || ttc >= tc_max) return d_min;
	if (ttc < tc_min) {
		double q = (double)((tc_min - ttc) / tc_min);
		return (float)(d_mid + q * q * (double)(d_max - d_mid));
	}
	if (ttc < tc_mid) return d_mid;
	return d_min + d_mid - (tc_max - ttc) / (tc_max - tc_mid);
}

static float cost_karamouzas(const actx* A, const up_cost* c, const cprep* P, v2 v)
{   /* Karamouzas.cpp:28-113 */
	const float alpha = c->p[0], beta = c->p[1], gamma = c->p[2], delta = c->p[3], t_max = c->p[4];
	const float tc_min = 2.5f, tc_max = 8;
	const float speed = vmag(v);
	const float ttcp = P->ttc_pref;
	if (vangle(v, A->pref) > karamouzas_maxdev(ttcp)) return MAXF;
	const float dS = fabsf(A->maxspeed - A->prefspeed), eps = 0.05f;
	float minS, maxS;
	if (ttcp <= 0 || ttcp >= tc_max) { minS = A->prefspeed - eps; maxS = A->prefspeed + eps; }
	else if (ttcp > 0 && ttcp < tc_min) { minS = 0; maxS = A->maxspeed + eps; }
	else { minS = A->prefspeed - dS - eps; maxS = A->prefspeed + dS + eps; }
	if (speed < minS || speed > maxS) return MAXF;
	float TTC = ttc_first(A, A->pos, v, A->radius, c->range, 1);
	float a = alpha * (1 - vcosangle(v, A->pref) / 2.0f);
	float b = beta * fabsf(speed - vmag(A->vel)) / A->maxspeed;
	float cc = gamma * vmag(vsub(v, A->pref)) / (2 * A->maxspeed);
	float d = delta * fmaxr(0.0f, t_max - TTC) / t_max;
	return a + b + cc + d;
}

static float cost_moussaid(const actx* A, const up_cost* c, v2 v)
{   /* Moussaid.cpp:28-62 */
	const float d_max = c->p[0];
	const float speed = vmag(v), prefSpeed = A->prefspeed;
	const v2 dir = vnorm(v);
	float ttc = ttc_first(A, A->pos, vmul(dir, prefSpeed), A->radius, c->range, 0);
	float DC = (ttc == MAXF ? MAXF : ttc * prefSpeed);
	if (DC > d_max) DC = d_max;
	float K = d_max * d_max + DC * DC - 2 * d_max * DC * vcosangle(dir, A->pref);
	K += 1;
	float S = fminr(prefSpeed, DC / A->relax);
	double q = (double)((S - speed) / S);
	return (float)(K * (1 + q * q));
}

static float cost_vantoll(const actx* A, const up_cost* c, v2 v)
{   /* VanToll.cpp:29-64 */
	const float maxd = c->p[0];
	const float prefSpeed = vmag(A->pref), speed = vmag(v);
	const float cTTC = ttc_first(A, A->pos, v, A->radius, c->range, 0);
	float dC = (cTTC == MAXF ? MAXF : cTTC * speed);
	if (dC > maxd) dC = maxd;
	const float a1 = vangle(v, A->pref);
	const float a2 = fabsf(speed - prefSpeed) / prefSpeed;
	const float a3 = vangle(v, A->vel);
	return 1 * (maxd - dC) + 1 * a1 + 1 * a2 + 1 * a3;
}

static float cost_pledestrians(const actx* A, const up_cost* c, v2 v)
{   /* PLEdestrians.cpp:28-36 */
	const float w_a = c->p[0], w_b = c->p[1], t_min = c->p[2], t_max = c->p[3];
	float ttc = ttc_first(A, A->pos, v, A->radius, c->range, 1);
	if (ttc < t_min) return MAXF;
	return t_max * (w_a + w_b * vsq(v)) + 2 * vmag(vsub(vsub(A->goal, A->pos), vmul(v, t_max))) * sqrtf(w_a * w_b);
}

static float cost_rvo(const actx* A, const up_cost* c, v2 v)
{   /* RVO.cpp:28-44 */
	if (vmag(v) > A->maxspeed) return MAXF;
	const v2 rv = vsub(vmul(v, 2), A->vel);
	const v2 vd = vsub(A->pref, v);
	float minT = ttc_first(A, A->pos, rv, A->radius, c->range, 1);
	return c->p[0] / minT + vmag(vd);
}

static float cost_orca(const actx* A, const cprep* P, v2 v)
{   /* ORCA.cpp:49-86 */
	float maxD = -MAXF;
	for (int k = 0; k < P->orca.nlines; ++k) {
		const v2 pm = vsub(P->orca.lines[k].point, v);
		maxD = fmaxr(maxD, P->orca.lines[k].dir.x * pm.y - P->orca.lines[k].dir.y * pm.x);
	}
	if (maxD <= 0) return vmag(vsub(v, A->pref));
	return maxD + 2 * A->maxspeed;
}

static float cost_paris(const actx* A, const up_cost* c, v2 v)
{   /* Paris.cpp:28-221 */
	const float w_a = c->p[0], w_b = c->p[1], t_max = c->p[2];
	const v2 dir = vnorm(v);
	const float rs = c->range * c->range;
	const float prefSpeed = vmag(A->pref);
	const float speed = vmag(v);
	float sumCP = 0, sumDev = 0;
	int cnt = 0;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 > rs) continue;
		const v2 np = e->pos, nv = A->w->vel[e->j];
		const float r1 = A->radius, r2 = A->w->radius[e->j];
		float t1, t2, s1, s2;
		v2 X;
		if (!line_intersection(A->pos, vadd(A->pos, dir), np, vadd(np, nv), &X)) {
			float ttc = ttc_pair(A->pos, dir, r1, np, nv, r2);
			if (ttc > t_max) { t1 = t_max; t2 = 0; s1 = 0; s2 = FLT_MAX; }
			else { t1 = 0; t2 = t_max; s1 = FLT_MAX; s2 = 0; }
		} else {
			/* ComputeT1andT2 for the agent (Paris.cpp:43-60) */
			float ta = ttc_pair(A->pos, A->vel, r1 + r2, X, V(0, 0), 0);
			if (ta > t_max) ta = t_max;
			if (ta == t_max) { t1 = t_max; t2 = 0; s1 = 0; s2 = FLT_MAX; }
			else {
				float u1 = ttc_pair(np, nv, r1 + r2, X, V(0, 0), 0);
				if (u1 > t_max) u1 = t_max;
				float u2 = u1 + (r1 + r2) / vmag(nv);
				if (u2 > t_max) u2 = 0;
				float distToX = vmag(vsub(X, A->pos));
				t1 = u1; t2 = u2;
				s1 = distToX / u1;
				s2 = distToX / u2;
			}
		}
		(void)t2;
		/* CSpeed * CPred (Paris.cpp:160-176) */
		float cs = fminr(fmaxr(0.0f, 1.0f - s1 / prefSpeed), fmaxr(0.0f, (s2 - prefSpeed) / prefSpeed));
		float cp = 1 - t1 / (t_max + w_b);
		sumCP += cs * cp;
		sumDev += fmaxr(0.0f, fmaxr((s1 - speed) / prefSpeed, (speed - s2) / prefSpeed));
		cnt++;
	}
	if (cnt > 0) sumCP /= (float)cnt;
	float cangle = (float)((1 - (double)vcosangle(dir, A->pref)) / 2.0);
	float dirCost = w_a * sumCP + (1 - w_a) * cangle;
	float diffToPref = vmag(vsub(v, A->pref));
	return 1000 * dirCost + sumDev + 0.001f * diffToPref;
}

static inline float ttcadca_pair_cost(float ttca, float dca, float sT, float sD)
{   /* TtcaDca.cpp:40-43 */
	double a = (double)(ttca / sT), b = (double)(dca / sD);
	return (float)exp(-0.5 * (a * a + b * b));
}

static float cost_ttcadca(const actx* A, const up_cost* c, v2 v)
{   /* TtcaDca.cpp:62-129 */
	const float sA = c->p[0], sS = c->p[1], sT = c->p[2], sD = c->p[3];
	const float viewHalf = (float)(REF_PI / 2.0);
	const float rs = c->range * c->range;
	/* getMovementCost: TtcaDca.cpp:45-52 */
	float alpha = vangle(v, A->pref);
	float ds = vmag(v) - A->prefspeed;
	double qa = (double)(alpha / sA), qs = (double)(ds / sS);
	float Ca = (float)exp(-0.5 * (qa * qa));
	float Cs = (float)exp(-0.5 * (qs * qs));
	float move = 1 - (Ca + Cs) / 2.0f;
	float oc = 0, sc = 0;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 >= rs) continue;
		const v2 relPos = vsub(e->pos, A->pos);
		if (vangle(relPos, A->vel) > viewHalf) continue;
		float ttca, dca;
		ttca_dca(A->pos, v, A->radius, e->pos, A->w->vel[e->j], A->w->radius[e->j], &ttca, &dca);
		float dist = vmag(relPos) - A->radius - A->w->radius[e->j];
		float scale = 1 / (dist * dist);
		sc += scale;
		float cost = ttcadca_pair_cost(ttca, dca, sT, sD) * scale;
		oc += cost;
	}
	if (sc > 0) oc /= sc;
	return oc + move;
}

static inline float foe_importance(float ttc)
{   /* FOEAvoidance.cpp:41-49 */
	if (ttc < 0.f || ttc > 10.f) return 0.f;
	float t0 = 5, I0 = 10, a = -I0 / t0;
	float I = a * ttc + I0;
	if (I < 0.1f) return 0.1f;
	if (I > 10.f) return 10.f;
	return I;
}

static float cost_foe(const actx* A, const up_cost* c, v2 v)
{   /* FOEAvoidance.cpp:50-92 */
	if (viszero(v)) return 0;
	const v2 Vn = vnorm(v);
	const float rs = c->range * c->range;
	float cost = 0;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 > rs) continue;
		v2 dv = vsub(A->w->vel[e->j], v), dp = vsub(e->pos, A->pos);
		/* RT = transpose of Matrix((Vn.y,-Vn.x), Vn) */
		v2 Vel = V(Vn.y * dv.x + -Vn.x * dv.y, Vn.x * dv.x + Vn.y * dv.y);
		v2 Pos = V(Vn.y * dp.x + -Vn.x * dp.y, Vn.x * dp.x + Vn.y * dp.y);
		if ((double)Pos.y < 0.1 || (double)Vel.y > -0.01) continue;
		float xf = Vel.x / Vel.y, xg = Pos.x / Pos.y, dx = xg - xf;
		float ttc = -Pos.y / Vel.y;
		float sigma = (float)((double)((A->radius + A->w->radius[e->j]) / Pos.y) / log(10.0));
		cost += foe_importance(ttc) * expf(-fabsf(dx) / sigma);
	}
	return cost;
}

static float cost_eval(const actx* A, const up_cost* c, cprep* P, v2 v)
{
	switch (c->kind) {
	case UP_SOCIALFORCES: case UP_POWERLAW: case UP_GOALREACHING:
		/* ForceBasedFunction::GetCost: ForceBasedFunction.cpp:26-30 */
		return 0.5f * vsq(vsub(v, P->target)) / A->dt;
	case UP_KARAMOUZAS: return cost_karamouzas(A, c, P, v);
	case UP_MOUSSAID: return cost_moussaid(A, c, v);
	case UP_VANTOLL: return cost_vantoll(A, c, v);
	case UP_PLEDESTRIANS: return cost_pledestrians(A, c, v);
	case UP_RVO: return cost_rvo(A, c, v);
	case UP_ORCA: return cost_orca(A, P, v);
	case UP_PARIS: return cost_paris(A, c, v);
	case UP_TTCADCA: return cost_ttcadca(A, c, v);
	case UP_FOE: return cost_foe(A, c, v);
	/* RandomFunction::GetCost: RandomFunction.cpp:25-28 (the agent's stream) */
	case UP_RANDOM: return rng_uniform(&((up_world*)A->w)->rng[A->i], -1, 1);
	case UP_GENERIC: return 0;   /* GenericCost::GetCost: GenericCost.cpp:27-31 */
	}
	return 0;
}

static void prepare(const actx* A, const up_cost* c, cprep* P)
{
	P->has_orca = 0;
	if (c->kind == UP_SOCIALFORCES || c->kind == UP_POWERLAW || c->kind == UP_GOALREACHING)
		P->target = target_velocity(A, c);
	else if (c->kind == UP_KARAMOUZAS)
		P->ttc_pref = ttc_first(A, A->pos, A->pref, A->radius, c->range, 1);
	else if (c->kind == UP_ORCA) {
		orca_solve(A, c, &P->orca);
		P->has_orca = 1;
	}
}

static void release(cprep* P)
{
	if (P->has_orca) { free(P->orca.lines); P->has_orca = 0; }
}

/* ------------------------------------------------------------------ */
/* gradients                                                           */
/* ------------------------------------------------------------------ */
static v2 grad_ttcadca(const actx* A, const up_cost* c, v2 v)
{   /* TtcaDca.cpp:131-262 */
	const float sA = c->p[0], sS = c->p[1], sT = c->p[2], sD = c->p[3];
	const float viewHalf = (float)(REF_PI / 2.0);
	const float eps = 0.001f;
	const float rs = c->range * c->range;
	float GradTh = 0, GradS = 0, total = 0;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 > rs) continue;
		const v2 dpc = vsub(e->pos, A->pos), dvc = vsub(A->w->vel[e->j], v);
		if (vangle(dpc, A->vel) > viewHalf) continue;
		float dpMag = vmag(dpc);
		const v2 dp = vmul(vdiv(dpc, dpMag), dpMag - A->radius - A->w->radius[e->j]);
		v2 nrm = V(-dpc.y, dpc.x);
		const v2 dv = vadd(dvc, vmul(nrm, vdot(nrm, dvc)));
		float dvSq = vsq(dv);
		float ttca = (dvSq == 0 ? 0 : -vdot(dp, dv) / dvSq);
		if (ttca < 0) ttca = 0;
		const v2 vdca = vadd(dp, vmul(dv, ttca));
		float dca = vmag(vdca);
		if (dca < 0) dca = 0;
		if (dvSq <= eps) continue;
		const v2 VelRot = V(dv.y, -dv.x);
		const float VelMag = sqrtf(dvSq);
		const v2 VelNorm = vdiv(dv, VelMag);
		float gTA = 0, gTS = 0;
		if (fabsf(ttca) > eps) {
			const v2 rel = vadd(dp, vmul(dv, 2 * ttca));
			gTA = -vdot(rel, VelRot) / dvSq;
			gTS = vdot(rel, VelNorm) / dvSq;
		}
		float gDA = 0, gDS = 0;
		if (fabsf(dca) > eps) {
			gDA = vdot(vdca, vadd(vmul(dv, gTA), vmul(VelRot, ttca))) / dca;
			gDS = vdot(vdca, vsub(vmul(dv, gTS), vmul(VelNorm, ttca))) / dca;
		}
		float cost = ttcadca_pair_cost(ttca, dca, sT, sD);
		float tf = ttca / (sT * sT), df = dca / (sD * sD);
		float gCS = -cost * (gTS * tf + gDS * df);
		float gCA = -cost * (gTA * tf + gDA * df);
		float scale = 1 / vsq(dp);
		total += scale;
		GradTh += gCA * scale;
		GradS += gCS * scale;
	}
	if (total > 0) { GradTh /= total; GradS /= total; }
	/* getMovementCostGradient: TtcaDca.cpp:54-60 */
	float alpha = vccwangle(v, A->pref);
	float ds = vmag(v) - A->prefspeed;
	double qa = (double)(alpha / sA), qs = (double)(ds / sS);
	double DCa = (double)(alpha / (2 * sA * sA)) * exp(-0.5 * (qa * qa));
	double DCs = (double)(ds / (2 * sS * sS)) * exp(-0.5 * (qs * qs));
	GradTh += (float)DCa;
	GradS += (float)DCs;
	if ((double)vsq(v) < 0.01)
		return rotate_gradient(GradTh, GradS, vnorm(A->pref), vmag(A->pref));
	return rotate_gradient(GradTh, GradS, vnorm(v), vmag(v));
}

static v2 grad_foe(const actx* A, const up_cost* c, v2 v)
{   /* FOEAvoidance.cpp:94-143 */
	if (viszero(v)) return V(0, 0);
	const v2 Vn = vnorm(v);
	const float rs = c->range * c->range;
	float gt = 0, gv = 0;
	for (int k = 0; k < A->L->n; ++k) {
		const nbr* e = &A->L->v[k];
		if (e->d2 > rs) continue;
		v2 dv = vsub(A->w->vel[e->j], v), dp = vsub(e->pos, A->pos);
		v2 Vel = V(Vn.y * dv.x + -Vn.x * dv.y, Vn.x * dv.x + Vn.y * dv.y);
		v2 Pos = V(Vn.y * dp.x + -Vn.x * dp.y, Vn.x * dp.x + Vn.y * dp.y);
		if ((double)Pos.y < 0.1 || (double)Vel.y > -0.01) continue;
		float xf = Vel.x / Vel.y, xg = Pos.x / Pos.y, dx = xg - xf;
		float ttc = -Pos.y / Vel.y;
		float sigma = (float)((double)((A->radius + A->w->radius[e->j]) / Pos.y) / log(10.0));
		float sg = (float)((0 < dx) - (dx < 0));
		float E = foe_importance(ttc) * expf(-fabsf(dx) / sigma);
		gt += E * sg * (xf * xf - xg * xg - (vmag(v) / (-Vel.y))) / sigma;
		gv += E * sg * (-xf / (-Vel.y)) / sigma;
	}
	if (gt < -0.1f) gt = -0.1f;
	else if (gt > 0.1f) gt = 0.1f;
	v2 w = vadd(vmul(V(sinf(gt), 1 - cosf(gt)), vmag(v)), V(0, gv));
	/* -1 * R * w with R = Matrix((Vn.y,-Vn.x), Vn) */
	return V(-Vn.y * w.x + -Vn.x * w.y, -(-Vn.x) * w.x + -Vn.y * w.y);
}

static v2 cost_gradient(const actx* A, const up_cost* c, cprep* P, v2 v)
{
	switch (c->kind) {
	case UP_SOCIALFORCES: case UP_POWERLAW: case UP_GOALREACHING:
		/* ForceBasedFunction::GetGradient: ForceBasedFunction.cpp:32-36 */
		return vdiv(vsub(v, P->target), A->dt);
	case UP_TTCADCA: return grad_ttcadca(A, c, v);
	case UP_FOE: return grad_foe(A, c, v);
	case UP_RANDOM: {
		/* RandomFunction::GetGradient: RandomFunction.cpp:30-33; the reference
		 * build evaluates the constructor's second argument first */
		uint32_t* st = &((up_world*)A->w)->rng[A->i];
		const float gy = rng_uniform(st, -1, 1);
		const float gx = rng_uniform(st, -1, 1);
		return V(gx, gy);
	}
	default: {
		/* CostFunction::GetGradient default: costFunction.cpp:36-54 */
		const float d = 0.1f;
		float cl = cost_eval(A, c, P, vsub(v, V(d, 0)));
		float cr = cost_eval(A, c, P, vadd(v, V(d, 0)));
		float gx = (cr - cl) / (2 * d);
		float cb = cost_eval(A, c, P, vsub(v, V(0, d)));
		float ct = cost_eval(A, c, P, vadd(v, V(0, d)));
		float gy = (ct - cb) / (2 * d);
		return V(gx, gy);
	}
	}
}

/* ------------------------------------------------------------------ */
/* optimisation methods (policy.cpp:43-105, costFunction.cpp:66-164)   */
/* ------------------------------------------------------------------ */
static v2 sample_min(actx* A, const up_policy* pol, int s_type, int s_base, int s_dir, int s_radius,
                     float s_angle, int nspeed, int nangle, int nrandom, int incl,
                     const up_cost* costs, const float* coeffs, int ncost, cprep* P)
{
	v2 base = V(0, 0);
	if (s_base == 1) base = A->vel;
	float radius = 0;
	if (s_radius == 0) radius = A->prefspeed;
	else if (s_radius == 1) radius = A->maxspeed;
	else radius = fminr(2.0f * A->maxspeed, A->maxacc * A->dt);
	v2 dir = V(1, 0);
	if (s_dir == 1) dir = vnorm(A->vel);
	else if (s_dir == 2) dir = vnorm(A->pref);
	float maxAngle = (float)(s_angle / 360.0 * REF_PI);
	v2 best = V(0, 0);
	float bestCost = MAXF;
	(void)pol;
	if (s_type == 1) {
		uint32_t* st = &((up_world*)A->w)->rng[A->i];
		for (int i = 0; i < nrandom; ++i) {
			float ra = rng_uniform(st, -maxAngle, maxAngle);
			float rl = rng_uniform(st, 0, radius);
			v2 v = vadd(base, vmul(vrot(dir, ra), rl));
			float tc = 0;
			for (int c = 0; c < ncost; ++c) tc += coeffs[c] * cost_eval(A, &costs[c], &P[c], v);
			if (tc < bestCost) { best = v; bestCost = tc; }
		}
	} else {
		const float start = -maxAngle, end = maxAngle;
		const float dA = (end - start) / (float)(s_angle == 360 ? nangle : (nangle - 1));
		const float dL = radius / (float)(incl ? (nspeed - 1) : nspeed);
		for (int s = 1; s <= nspeed; ++s) {
			const float len = dL * (float)(incl ? s - 1 : s);
			float ang = start;
			for (int a = 0; a < nangle; ++a, ang += dA) {
				v2 v = vadd(base, vmul(vrot(dir, ang), len));
				float tc = 0;
				for (int c = 0; c < ncost; ++c) tc += coeffs[c] * cost_eval(A, &costs[c], &P[c], v);
				if (tc < bestCost) { best = v; bestCost = tc; }
				if (incl && s == 1) break;
			}
		}
	}
	return best;
}

static v2 new_velocity(actx* A, const up_policy* pol)
{   /* Policy::ComputeNewVelocity: policy.cpp:43-76 */
	if (viszero(A->pref)) return V(0, 0);
	const v2 cur = A->vel;
	const float dt = A->dt;
	cprep P[UP_MAX_COSTS];
	float coeffs[UP_MAX_COSTS];
	for (int c = 0; c < pol->ncost; ++c) { prepare(A, &pol->cost[c], &P[c]); coeffs[c] = pol->cost[c].coeff; }
	v2 acc;
	if (pol->method == UP_GRADIENT) {
		v2 T = V(0, 0);   /* policy.cpp:78-89 */
		for (int c = 0; c < pol->ncost; ++c) {
			v2 g = cost_gradient(A, &pol->cost[c], &P[c], cur);
			T = vadd(T, vmul(g, pol->cost[c].coeff));
		}
		acc = vmul(T, -1);
	} else {
		v2 best;
		if (pol->method == UP_GLOBAL && pol->ncost == 1) {
			const up_cost* c0 = &pol->cost[0];
			if (c0->kind == UP_ORCA) best = P[0].orca.velocity;
			else if (c0->kind == UP_SOCIALFORCES || c0->kind == UP_POWERLAW || c0->kind == UP_GOALREACHING)
				best = P[0].target;
			else {  /* CostFunction::GetGlobalMinimum default: costFunction.cpp:56-64 */
				float one = 1.0f;
				best = sample_min(A, pol, 0, 0, 0, 1, 360, 11, 36, 0, 1, c0, &one, 1, P);
			}
		} else if (pol->method == UP_GLOBAL) {
			/* policy.cpp:91-100: ApproximateGlobalOptimization sampling */
			best = sample_min(A, pol, 0, 0, 0, 1, 360, 11, 36, 0, 1, pol->cost, coeffs, pol->ncost, P);
		} else {
			best = sample_min(A, pol, pol->s_type, pol->s_base, pol->s_dir, pol->s_radius, pol->s_angle,
			                  pol->speed_samples, pol->angle_samples, pol->random_samples, pol->include_base,
			                  pol->cost, coeffs, pol->ncost, P);
		}
		acc = vdiv(vsub(best, cur), fmaxr(pol->relax_time, dt));
	}
	for (int c = 0; c < pol->ncost; ++c) release(&P[c]);
	acc = vclamp(acc, A->maxacc);
	return vclamp(vadd(cur, vmul(acc, dt)), A->maxspeed);
}

static v2 contact_forces(const actx* A, const up_policy* pol)
{   /* Policy::ComputeContactForces: policy.cpp:107-141 */
	v2 total = V(0, 0);
	if (pol->contact_scale > 0) {
		for (int k = 0; k < A->L->n; ++k) {
			const nbr* e = &A->L->v[k];
			const v2 diff = vsub(A->pos, e->pos);
			const float inter = A->radius + A->w->radius[e->j] - vmag(diff);
			if (inter > 0) total = vadd(total, vmul(vnorm(diff), pol->contact_scale * inter));
		}
		/* colliding obstacles: policy.cpp:126-137 */
		for (int k = 0; k < A->O->n; ++k) {
			const seg e = A->O->v[k];
			const v2 diff = vsub(A->pos, nearest_on_segment(A->pos, e.a, e.b));
			const float inter = A->radius - vmag(diff);
			if (inter > 0) total = vadd(total, vmul(vnorm(diff), pol->contact_scale * inter));
		}
	}
	return total;
}

static void make_ctx(up_world* w, int i, actx* A)
{
	A->w = w; A->i = i; A->L = &w->nb[i]; A->O = &w->ob[i];
	A->pos = w->pos[i]; A->vel = w->vel[i]; A->pref = w->pref[i]; A->goal = w->goal[i];
	A->radius = w->radius[i]; A->prefspeed = w->prefspeed[i]; A->maxspeed = w->maxspeed[i];
	A->maxacc = w->maxacc[i]; A->dt = w->dt; A->relax = w->pol[w->policy[i]].relax_time;
}

/* the slot state of a new agent (Agent constructor, setPosition, setGoal:
 * agent.cpp:29-47, 108-115) */
static void init_slot(up_world* w, int i, long long id, v2 pos, v2 goal, float radius, float prefspeed,
                      float maxspeed, float maxacc, int policy)
{
	w->id[i] = id;
	w->pos[i] = pos;
	w->goal[i] = goal;
	w->radius[i] = radius; w->prefspeed[i] = prefspeed;
	w->maxspeed[i] = maxspeed; w->maxacc[i] = maxacc;
	w->policy[i] = policy;
	w->rng[i] = minstd_seed((uint64_t)(unsigned int)id);
	w->vel[i] = w->vwf[i] = w->pref[i] = w->next[i] = w->contact[i] = V(0, 0);
	w->view[i] = V(0, 0);
	if (goal.x != pos.x || goal.y != pos.y) w->view[i] = vnorm(vsub(goal, pos));
	w->nb[i].n = 0;
	w->ob[i].n = 0;
}

/* WorldBase::removeAgentAtListIndex: worldBase.cpp:207-235 (the last agent
 * moves into the freed slot); the slots' list buffers are swapped */
static void remove_slot(up_world* w, int i)
{
	const int last = w->n - 1;
	if (i != last) {
		w->id[i] = w->id[last];
		v2* vs[] = { w->pos, w->vel, w->goal, w->pref, w->next, w->vwf, w->view, w->contact };
		for (int k = 0; k < 8; ++k) vs[k][i] = vs[k][last];
		float* fs[] = { w->radius, w->prefspeed, w->maxspeed, w->maxacc };
		for (int k = 0; k < 4; ++k) fs[k][i] = fs[k][last];
		w->policy[i] = w->policy[last];
		w->rng[i] = w->rng[last];
		if (w->rmg) w->rmg[i] = w->rmg[last];
		nbrlist t = w->nb[i]; w->nb[i] = w->nb[last]; w->nb[last] = t;
		seglist u = w->ob[i]; w->ob[i] = w->ob[last]; w->ob[last] = u;
	}
	w->n = last;
}

static void do_step(up_world* w)
{   /* WorldBase::DoStep: worldBase.cpp:79-128 */
	/* agents whose start time has come join the end of the list */
	while (w->next_pend < w->npend && (double)w->pend[w->next_pend].start <= w->time) {
		const struct up_pending* a = &w->pend[w->next_pend++];
		const int i = w->n++;
		init_slot(w, i, a->id, a->pos, a->goal, a->radius, a->prefspeed, a->maxspeed, a->maxacc, a->policy);
		if (w->rmg) w->rmg[i] = a->rmg;
	}
	const int n = w->n;
	grid_build(w);
#pragma omp parallel for schedule(dynamic, 64)
	for (int i = 0; i < n; ++i) compute_neighbors(w, i);
#pragma omp parallel for schedule(static)
	for (int i = 0; i < n; ++i) {   /* Agent::ComputePreferredVelocity: agent.cpp:52-59 */
		v2 d = vsub(w->goal[i], w->pos[i]);
		if (vsq(d) <= w->radius[i] * w->radius[i]) w->pref[i] = V(0, 0);
		else w->pref[i] = vmul(vnorm(d), w->prefspeed[i]);
	}
#pragma omp parallel for schedule(dynamic, 16)
	for (int i = 0; i < n; ++i) {
		actx A;
		make_ctx(w, i, &A);
		w->next[i] = new_velocity(&A, &w->pol[w->policy[i]]);
	}
#pragma omp parallel for schedule(dynamic, 64)
	for (int i = 0; i < n; ++i) {
		actx A;
		make_ctx(w, i, &A);
		w->contact[i] = contact_forces(&A, &w->pol[w->policy[i]]);
	}
	const float hw = 0.5f * w->width, hh = 0.5f * w->height;
#pragma omp parallel for schedule(static)
	for (int i = 0; i < n; ++i) {   /* Agent::UpdateVelocityAndPosition: agent.cpp:71-93 */
		w->vwf[i] = w->next[i];
		const v2 af = vdiv(w->contact[i], 80.0f);
		w->vel[i] = vadd(w->vwf[i], vmul(af, w->dt));
		const v2 vd = vdiv(vadd(vmul(w->vel[i], 2), w->pref[i]), 3);
		if ((double)vsq(vd) > 0.01) w->view[i] = vnorm(vd);
		w->pos[i] = vadd(w->pos[i], vmul(w->vel[i], w->dt));
		if (w->type == UP_TORIC) {   /* worldToric.cpp:81-108 */
			float x = w->pos[i].x, y = w->pos[i].y;
			if (x > hw) x -= w->width;
			else if (x < -hw) x += w->width;
			if (y > hh) y -= w->height;
			else if (y < -hh) y += w->height;
			w->pos[i] = V(x, y);
		}
	}
	w->time += w->dt;
	/* agents at their goal that are to be removed there, from the back */
	if (w->rmg)
		for (int i = n - 1; i >= 0; --i)
			if (w->rmg[i] && vsq(vsub(w->goal[i], w->pos[i])) <= w->radius[i] * w->radius[i]) remove_slot(w, i);
}

/* ------------------------------------------------------------------ */
/* API                                                                 */
/* ------------------------------------------------------------------ */
up_world* up_create(int n, int world_type, float width, float height, float dt,
                    const up_policy* policies, int npolicies,
                    const long long* ids, const float* pos, const float* goal,
                    const float* radius, const float* pref_speed, const float* max_speed,
                    const float* max_accel, const int* policy_index)
{
	up_world* w = (up_world*)calloc(1, sizeof(up_world));
	w->n = n; w->type = world_type; w->width = width; w->height = height; w->dt = dt;
	w->npol = npolicies;
	w->pol = (up_policy*)malloc(sizeof(up_policy) * (size_t)(npolicies > 0 ? npolicies : 1));
	memcpy(w->pol, policies, sizeof(up_policy) * (size_t)npolicies);
	size_t N = (size_t)(n > 0 ? n : 1);
	w->id = (long long*)malloc(sizeof(long long) * N);
	v2** vs[] = { &w->pos, &w->vel, &w->goal, &w->pref, &w->next, &w->vwf, &w->view, &w->contact };
	for (int k = 0; k < 8; ++k) *vs[k] = (v2*)calloc(N, sizeof(v2));
	float** fs[] = { &w->radius, &w->prefspeed, &w->maxspeed, &w->maxacc };
	for (int k = 0; k < 4; ++k) *fs[k] = (float*)calloc(N, sizeof(float));
	w->policy = (int*)calloc(N, sizeof(int));
	w->rng = (uint32_t*)calloc(N, sizeof(uint32_t));
	w->nb = (nbrlist*)calloc(N, sizeof(nbrlist));
	w->ob = (seglist*)calloc(N, sizeof(seglist));
	for (int i = 0; i < n; ++i) {
		w->id[i] = ids[i];
		w->pos[i] = V(pos[2 * i], pos[2 * i + 1]);
		w->goal[i] = V(goal[2 * i], goal[2 * i + 1]);
		w->radius[i] = radius[i]; w->prefspeed[i] = pref_speed[i];
		w->maxspeed[i] = max_speed[i]; w->maxacc[i] = max_accel[i];
		w->policy[i] = policy_index[i];
		w->rng[i] = minstd_seed((uint64_t)(unsigned int)ids[i]);
		/* Agent::setGoal: agent.cpp:108-115 */
		if (w->goal[i].x != w->pos[i].x || w->goal[i].y != w->pos[i].y)
			w->view[i] = vnorm(vsub(w->goal[i], w->pos[i]));
	}
	return w;
}

void up_free(up_world* w)
{
	if (!w) return;
	const int slots = w->cap > w->n ? w->cap : w->n;
	for (int i = 0; i < slots; ++i) { free(w->nb[i].v); free(w->ob[i].v); }
	free(w->rmg); free(w->pend);
	free(w->nb); free(w->ob); free(w->edges); free(w->pol); free(w->id);
	free(w->pos); free(w->vel); free(w->goal); free(w->pref); free(w->next); free(w->vwf);
	free(w->view); free(w->contact); free(w->radius); free(w->prefspeed); free(w->maxspeed);
	free(w->maxacc); free(w->policy); free(w->rng); free(w->cell_start); free(w->cell_items);
	free(w);
}

void up_set_obstacles(up_world* w, int ne, const float* edges)
{   /* WorldBase::AddObstacle (worldBase.cpp:239-242): edges (ax, ay, bx, by) */
	free(w->edges);
	w->ne = ne;
	w->edges = (seg*)malloc(sizeof(seg) * (size_t)(ne > 0 ? ne : 1));
	for (int k = 0; k < ne; ++k) {
		w->edges[k].a = V(edges[4 * k], edges[4 * k + 1]);
		w->edges[k].b = V(edges[4 * k + 2], edges[4 * k + 3]);
	}
}

void up_set_dynamics(up_world* w, const float* start_time, const unsigned char* remove_at_goal)
{   /* WorldBase::AddAgent (worldBase.cpp:161-188) at time 0: an agent with a
	 * start time > 0 waits in the insertion queue, the others form the list */
	w->cap = w->n;
	w->rmg = (unsigned char*)calloc((size_t)(w->n > 0 ? w->n : 1), 1);
	w->pend = (struct up_pending*)malloc(sizeof(struct up_pending) * (size_t)(w->n > 0 ? w->n : 1));
	w->npend = w->next_pend = 0;
	int m = 0;
	for (int i = 0; i < w->n; ++i) {
		const float st = start_time ? start_time[i] : 0.0f;
		const unsigned char rg = remove_at_goal ? remove_at_goal[i] : 0;
		if ((double)st <= w->time) {
			init_slot(w, m, w->id[i], w->pos[i], w->goal[i], w->radius[i], w->prefspeed[i], w->maxspeed[i],
			          w->maxacc[i], w->policy[i]);
			w->rmg[m++] = rg;
		} else {
			struct up_pending* a = &w->pend[w->npend++];
			a->id = w->id[i]; a->pos = w->pos[i]; a->goal = w->goal[i];
			a->radius = w->radius[i]; a->prefspeed = w->prefspeed[i]; a->maxspeed = w->maxspeed[i];
			a->maxacc = w->maxacc[i]; a->policy = w->policy[i]; a->start = st; a->rmg = rg;
		}
	}
	w->n = m;
	/* stable insertion sort by start time (equal times keep file order) */
	for (int i = 1; i < w->npend; ++i) {
		struct up_pending a = w->pend[i];
		int j = i - 1;
		while (j >= 0 && w->pend[j].start > a.start) { w->pend[j + 1] = w->pend[j]; --j; }
		w->pend[j + 1] = a;
	}
}

int up_num_agents(const up_world* w) { return w->n; }
double up_time(const up_world* w) { return w->time; }

double up_step(up_world* w, int n, int threads)
{
	if (threads > 0) omp_set_num_threads(threads);
	double t0 = omp_get_wtime();
	for (int s = 0; s < n; ++s) do_step(w);
	return omp_get_wtime() - t0;
}

void up_state(const up_world* w, long long* ids, float* pos, float* vel,
              float* prefvel, float* viewdir, float* goal)
{
	for (int i = 0; i < w->n; ++i) {
		if (ids) ids[i] = w->id[i];
		if (pos) { pos[2 * i] = w->pos[i].x; pos[2 * i + 1] = w->pos[i].y; }
		if (vel) { vel[2 * i] = w->vel[i].x; vel[2 * i + 1] = w->vel[i].y; }
		if (prefvel) { prefvel[2 * i] = w->pref[i].x; prefvel[2 * i + 1] = w->pref[i].y; }
		if (viewdir) { viewdir[2 * i] = w->view[i].x; viewdir[2 * i + 1] = w->view[i].y; }
		if (goal) { goal[2 * i] = w->goal[i].x; goal[2 * i + 1] = w->goal[i].y; }
	}
}

void up_set_state(up_world* w, const float* pos, const float* vel, const float* viewdir)
{   /* SetAgentPositions: APIFunctions.cpp:117-137 */
	for (int i = 0; i < w->n; ++i) {
		if (pos) w->pos[i] = V(pos[2 * i], pos[2 * i + 1]);
		if (vel) { w->vel[i] = V(vel[2 * i], vel[2 * i + 1]); w->vwf[i] = w->vel[i]; }
		if (viewdir) w->view[i] = V(viewdir[2 * i], viewdir[2 * i + 1]);
	}
}

/* the host C library's expf over an array (checks the device exponential) */
void up_libm_expf(const float* x, float* y, long n)
{
	for (long i = 0; i < n; ++i) y[i] = expf(x[i]);
}

void up_libm_sincosf(const float* x, float* s, float* c, long n)
{
	for (long i = 0; i < n; ++i) { s[i] = sinf(x[i]); c[i] = cosf(x[i]); }
}

int up_neighbors(const up_world* w, int i, long long* ids, float* dist2, float* px, float* py, int cap)
{
	const nbrlist* L = &w->nb[i];
	for (int k = 0; k < L->n && k < cap; ++k) {
		ids[k] = w->id[L->v[k].j];
		dist2[k] = L->v[k].d2;
		px[k] = L->v[k].pos.x;
		py[k] = L->v[k].pos.y;
	}
	return L->n;
}
