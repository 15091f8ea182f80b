// Plain-data descriptors shared by the host loader and the device kernels.
//
// A policy is the reference's Policy (src/Engine/core/policy.h:127-181): an
// optimisation method, sampling parameters (policy.h:36-87), a relaxation
// time, a contact-force scale and a list of weighted cost functions.  Each
// cost function is one of the reference's registered CostFunction plugins
// (src/Engine/core/costFunctionFactory.cpp:41-61), identified by kind, with
// its range, coefficient and model parameters.
#pragma once
#include <cmath>
#include <cstdint>

namespace umans {

enum CostKind : int {
	K_ORCA = 0, K_RVO, K_SOCIALFORCES, K_POWERLAW, K_GOALREACHING, K_KARAMOUZAS,
	K_MOUSSAID, K_PARIS, K_VANTOLL, K_TTCADCA, K_FOE, K_PLEDESTRIANS, K_RANDOM, K_GENERIC, K_NUM_KINDS,
	K_PLUGIN0 = K_NUM_KINDS   // cost-function plugins: K_PLUGIN0 + index in kPlugins (plugins.hpp)
};
enum Method : int { M_GRADIENT = 0, M_SAMPLING = 1, M_GLOBAL = 2 };
enum WorldType : int { W_INFINITE = 0, W_TORIC = 1 };

constexpr int MAX_COSTS = 4;

struct CostDesc {
	int kind;
	float coeff;
	float range;
	// model parameters by kind (defaults from the reference headers):
	//  ORCA p0 timeHorizon | RVO p0 w
	//  SocialForcesAvoidance p0 dt, p1 V0, p2 sigma, p3 U0, p4 R, p5 agentMass
	//  PowerLaw p0 k, p1 tau0, p5 agentMass | GoalReachingForce p5 agentMass
	//  Karamouzas p0 alpha, p1 beta, p2 gamma, p3 delta, p4 t_max
	//  Moussaid p0 d_max | Paris p0 w_a, p1 w_b, p2 t_max | VanToll p0 max_distance
	//  TtcaDca p0 sigAngle_goal, p1 sigSpeed_goal, p2 sigTtca, p3 sigDca
	//  PLEdestrians p0 w_a, p1 w_b, p2 t_min, p3 t_max
	float p[8];
};

// Regular-sampling schedule (costFunction.cpp:122-158): the float angle
// sequence is agent independent, so (cosf, sinf) of every candidate angle and
// the speed multiplier (s-1 or s) are tabulated on the host.
struct SampleEntry { float c, s, mult, pad; };

struct PolicyDesc {
	int method;
	int s_type;      // 0 regular, 1 random
	int s_base;      // 0 zero, 1 current velocity
	int s_dir;       // 0 unit, 1 current velocity, 2 preferred velocity
	int s_radius;    // 0 preferred speed, 1 maximum speed, 2 maximum acceleration
	float s_angle;   // full sampled angle in degrees
	int speed_samples, angle_samples, random_samples, include_base;
	float relax_time;
	float contact_scale;
	float max_angle;     // (float)(s_angle / 360.0 * PI)
	float range;         // Policy::getInteractionRange (policy.cpp:34-41)
	int ncost;
	CostDesc cost[MAX_COSTS];
	// derived: how the velocity is chosen this step
	int use_sampling;    // 1 when a sample table drives the choice
	int table_offset;    // into the sample-table buffer
	int nsamples;        // regular: table entries; random: random_samples
	int len_divisor;     // regular: speed_samples - 1 or speed_samples
	int table_radius;    // radius rule of the table actually used
	int table_dir;       // direction rule of the table actually used
	int table_base;      // base rule of the table actually used
	int table_random;    // 1 when random sampling is used
	int single_cost;     // GLOBAL with one non-closed-form cost: sample only cost[0] with coeff 1
	int nrand;           // RandomFunction costs among the ones evaluated per sample / gradient
	int draws;           // random numbers drawn per sample (random sampling: 2, + nrand)
};

// Same layout as the C ABI's struct AgentData (28 bytes).
struct AgentRecord {
	int id;
	float px, py, vx, vy, wx, wy;
};

// One scenario of a simulation (a batch holds several, agents concatenated).
struct ScenDesc {
	int world;
	float width, height, dt;
	float max_range;      // largest interaction range of its policies
	int agent_off, n;     // its agents occupy list slots [agent_off, agent_off + n)
	int max_cells;        // cap on its grid's cell count
	int edge_off, nedges; // its obstacle edges in the concatenated edge array
	// uniform grid over its edges (og_nx == 0: none, the edges are scanned):
	// cell (cx, cy) holds the edges whose bounding box overlaps it, as items
	// [og_start + start[cy * og_nx + cx], ...) of the engine's item arrays
	float og_x0, og_y0, og_inv;
	int og_nx, og_ny, og_start;
};

// scenarios with at least this many edges get an edge grid
constexpr int OBS_GRID_MIN_EDGES = 256;

// cell coordinate along one axis, the same on the host and the device
#if defined(__CUDACC__)
__host__ __device__
#endif
inline int obs_cell(float v, float v0, float inv, int n)
{
	const float f = (v - v0) * inv;
	int c = (f >= 0.0f) ? (int)fminf(f, 2.0e9f) : 0;   // NaN -> 0
	return c >= n ? n - 1 : c;
}

// Grid parameters written by the device each step.
struct GridParams {
	float x0, y0, cs, inv_cs;
	int nx, ny, ncells, pad;
};

// status bits reported by the device
enum StatusBits : int {
	ST_NEIGHBOUR_OVERFLOW = 1,
	ST_ORCA_OVERFLOW = 2,
	ST_GRID_OVERFLOW = 4,
	ST_GRID_BARRIER = 8,   // a grid barrier of the one-launch grid build gave up waiting
};

}  // namespace umans
