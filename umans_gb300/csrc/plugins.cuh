// Device side of the cost-function plugins (plugins.hpp): one function per
// entry of kPlugins, dispatched by index.
#pragma once
#include "costs.cuh"
#include "plugins.hpp"

namespace umans {

// ExampleRVO (kPlugins[0]): RVO::GetCost, RVO.cpp:28-44
__device__ __forceinline__ float plugin_example_rvo(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	if (vmag(v) > A.maxspeed) return MAXF;
	const float2 rv = vsub(vmul(v, 2), A.vel);
	const float2 vd = vsub(A.pref, v);
	const float minT = ttc_first(A, N, rv, c.range, true);
	return c.p[0] / minT + vmag(vd);
}

// ExampleFOE (kPlugins[1]): FOEAvoidance::GetCost (FOEAvoidance.cpp:50-92)
// and its closed-form GetGradient (:94-143), through the engine's own
// restatements of both
__device__ __forceinline__ float plugin_example_foe(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	return cost_foe(A, N, c, v);
}
__device__ __forceinline__ float2 plugin_example_foe_gradient(const AgentCtx& A, const NbView& N, const CostDesc& c,
                                                              float2 v, int lane, float* z0, float* z1)
{
	return grad_foe(A, N, c, v, lane, z0, z1);
}

// ExampleGoal (kPlugins[2]): GoalReachingForce as a ForceBasedFunction.
// target = v + F / agentMass dt with F = (v_pref - v) / max(relax, dt)
// (ForceBasedFunction.cpp:48-52, GoalReachingForce.cpp:26-29); cost
// 0.5 |v - target|^2 / dt, gradient (v - target) / dt, global minimum
// target (ForceBasedFunction.cpp:26-40)
__device__ __forceinline__ float2 example_goal_target(const AgentCtx& A, const CostDesc& c)
{
	const float2 F = vdiv(vsub(A.pref, A.vel), fmaxr(A.relax, A.dt));
	return vadd(A.vel, vmul(vdiv(F, c.p[5]), A.dt));
}
__device__ __forceinline__ float plugin_example_goal(const AgentCtx& A, const NbView&, const CostDesc& c, float2 v)
{
	return 0.5f * vsq(vsub(v, example_goal_target(A, c))) / A.dt;
}

static_assert(kPluginCount == 3, "plugin_cost, plugin_gradient and plugin_global_minimum need one case per plugin");

__device__ __forceinline__ float plugin_cost(int index, const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	switch (index) {
	case 0: return plugin_example_rvo(A, N, c, v);
	case 1: return plugin_example_foe(A, N, c, v);
	case 2: return plugin_example_goal(A, N, c, v);
	}
	return 0;
}

// GetGradient overrides: true with *g set when plugin `index` has one
__device__ __forceinline__ bool plugin_gradient(int index, const AgentCtx& A, const NbView& N, const CostDesc& c,
                                                float2 v, int lane, float* z0, float* z1, float2* g)
{
	switch (index) {
	case 1: *g = plugin_example_foe_gradient(A, N, c, v, lane, z0, z1); return true;
	case 2: *g = vdiv(vsub(v, example_goal_target(A, c)), A.dt); return true;
	}
	return false;
}

// GetGlobalMinimum overrides: true with *best set when plugin `index` has one
__device__ __forceinline__ bool plugin_global_minimum(int index, const AgentCtx& A, const NbView& N, const CostDesc& c,
                                                      int lane, float2* best)
{
	switch (index) {
	case 2: *best = example_goal_target(A, c); return true;
	}
	return false;
}

}  // namespace umans
