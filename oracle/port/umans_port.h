/* CPU restatement of the UMANS per-step agent update (WorldBase::DoStep).
 *
 * TEST INFRASTRUCTURE: this is the oracle.  Only tests, the golden-fixture
 * tooling and the CPU-baseline leg of bench.py use it; the product never
 * links or calls it.  Each function in umans_port.c cites the reference
 * file:line it restates.
 *
 * Parity pin: the port is checked against the reference engine compiled from
 * its own sources (oracle/_ref) on the example scenarios and the seeded
 * workloads, and against the golden trajectories under tests/golden/.
 */
#ifndef UMANS_PORT_H
#define UMANS_PORT_H

#ifdef __cplusplus
extern "C" {
#endif

/* cost-function kinds; names as registered in costFunctionFactory.cpp:41-61 */
enum up_cost_kind {
	UP_ORCA = 0, UP_RVO, UP_SOCIALFORCES, UP_POWERLAW, UP_GOALREACHING,
	UP_KARAMOUZAS, UP_MOUSSAID, UP_PARIS, UP_VANTOLL, UP_TTCADCA,
	UP_FOE, UP_PLEDESTRIANS, UP_RANDOM, UP_GENERIC, UP_NUM_KINDS
};
enum up_method { UP_GRADIENT = 0, UP_SAMPLING = 1, UP_GLOBAL = 2 };
enum up_world_type { UP_INFINITE = 0, UP_TORIC = 1 };

#define UP_MAX_COSTS 8
#define UP_MAX_PARAMS 8

typedef struct {
	int kind;
	float coeff;
	float range;
	/* model parameters, per kind (defaults from the reference headers):
	 *  ORCA:          p0 timeHorizon
	 *  RVO:           p0 w
	 *  SocialForces:  p0 dt, p1 V0, p2 sigma, p3 U0, p4 R, p5 agentMass
	 *  PowerLaw:      p0 k, p1 tau0, p5 agentMass
	 *  GoalReaching:  p5 agentMass
	 *  Karamouzas:    p0 alpha, p1 beta, p2 gamma, p3 delta, p4 t_max
	 *  Moussaid:      p0 d_max
	 *  Paris:         p0 w_a, p1 w_b, p2 t_max
	 *  VanToll:       p0 max_distance
	 *  TtcaDca:       p0 sigAngle_goal, p1 sigSpeed_goal, p2 sigTtca, p3 sigDca
	 *  PLEdestrians:  p0 w_a, p1 w_b, p2 t_min, p3 t_max */
	float p[UP_MAX_PARAMS];
} up_cost;

typedef struct {
	int method;
	/* SamplingParameters (policy.h:36-87) */
	int s_type;          /* 0 regular, 1 random */
	int s_base;          /* 0 zero, 1 current velocity */
	int s_dir;           /* 0 unit, 1 current velocity, 2 preferred velocity */
	int s_radius;        /* 0 preferred speed, 1 maximum speed, 2 maximum acceleration */
	float s_angle;
	int speed_samples, angle_samples, random_samples, include_base;
	float relax_time;
	float contact_scale;
	int ncost;
	up_cost cost[UP_MAX_COSTS];
} up_policy;

typedef struct up_world up_world;

up_world* up_create(int n, int world_type, float width, float height, float dt,
                    const up_policy* policies, int npolicies,
                    const long long* ids, const float* pos, const float* goal,
                    const float* radius, const float* pref_speed, const float* max_speed,
                    const float* max_accel, const int* policy_index);
void up_free(up_world* w);
/* static obstacle edges (ax, ay, bx, by), in file order */
void up_set_obstacles(up_world* w, int ne, const float* edges);
/* timed insertion and remove-at-goal (per agent, in creation order; either
 * may be NULL); call once, right after up_create */
void up_set_dynamics(up_world* w, const float* start_time, const unsigned char* remove_at_goal);
int up_num_agents(const up_world* w);
double up_time(const up_world* w);
/* runs n steps with `threads` OpenMP threads; returns wall seconds */
double up_step(up_world* w, int n, int threads);
void up_state(const up_world* w, long long* ids, float* pos, float* vel,
              float* prefvel, float* viewdir, float* goal);
void up_set_state(up_world* w, const float* pos, const float* vel, const float* viewdir);
/* neighbour list agent i used in the last step (reference order) */
int up_neighbors(const up_world* w, int i, long long* ids, float* dist2,
                 float* px, float* py, int cap);

void up_libm_expf(const float* x, float* y, long n);
/* the host C library's sinf / cosf (test reference of the device's) */
void up_libm_sincosf(const float* x, float* s, float* c, long n);

#ifdef __cplusplus
}
#endif
#endif
