// Cost-function plugins: the engine's counterpart of the reference's
// CostFunction plugin API (src/Engine/core/costFunction.h:155-194: GetCost,
// parseParameters, GetName; registration with registerCostFunction<T>(),
// src/Engine/core/costFunctionFactory.h:44-53 and .cpp:41-61).
//
// A plugin has two parts, both added to the library at build time:
//  * a host table entry below (kPlugins in plugins.cpp): the name a
//    <costfunction name="..."/> element uses (GetName), and its parameters:
//    XML attribute, slot in CostDesc::p, default (parseParameters); `range`
//    and `coeff` are read for every cost function;
//  * a device function in plugins.cuh, dispatched by plugin_cost():
//      __device__ float cost(const AgentCtx& A, const NbView& N,
//                            const CostDesc& c, float2 v);   // GetCost
//    with the agent (A), its neighbour and obstacle lists (N) and the
//    candidate velocity v, using the helpers of costs.cuh (time to first
//    collision, closest approach, ...) and the host-exact libm functions
//    (ref_expf(A.ex, x), host_sinf, host_sincosf), whose tables the engine
//    uploads for every scenario with a plugin cost;
//  * optionally, the overrides of the reference's virtual GetGradient
//    (costFunction.h:165) and GetGlobalMinimum (costFunction.h:173),
//    dispatched by plugin_gradient() and plugin_global_minimum():
//      __device__ float2 gradient(const AgentCtx& A, const NbView& N,
//                                 const CostDesc& c, float2 v, int lane,
//                                 float* z0, float* z1);
//      __device__ float2 global_minimum(const AgentCtx& A, const NbView& N,
//                                       const CostDesc& c, int lane);
//    called by the whole warp (lane = this lane; z0, z1: the warp's
//    per-neighbour scratch, N.K floats each).  The gradient method takes a
//    plugin's gradient where it has one, else the reference's default
//    finite difference (costFunction.cpp:36-54); the global method with a
//    plugin as its only cost takes its global minimum where it has one, else
//    the default sampling (policy.h:74-86, costFunction.cpp:56-64).
// A plugin cost is evaluated inside the agent kernel like the built-in
// per-sample costs: on every candidate of the sampling method, through the
// default sampling of the global method (policy.h:74-86), and through the
// default finite-difference gradient (costFunction.cpp:36-54) of the
// gradient method.  Its kind is K_PLUGIN0 + its index in kPlugins.
#pragma once

namespace umans {

struct PluginParam {
	const char* attr;   // XML attribute
	int slot;           // CostDesc::p index (0..7, checked at compile time in plugins.cpp)
	float dflt;         // default value
};

struct PluginInfo {
	const char* name;
	const PluginParam* params;
	int nparams;
	float range;        // default range (the plugin's constructor), < 0: CostFunction's 5 m
	bool gradient;      // overrides GetGradient (plugin_gradient has its case)
	bool global_minimum;  // overrides GetGlobalMinimum (plugin_global_minimum has its case)
};

// the number of plugins: the length of kPlugins and the number of cases of
// plugin_cost (plugins.cuh), both checked against it at compile time
constexpr int kPluginCount = 3;

extern const PluginInfo kPlugins[];
extern const int kNumPlugins;

}  // namespace umans
