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

static_assert(kPluginCount == 1, "plugin_cost needs one case per plugin: update both");

__device__ __forceinline__ float plugin_cost(int index, const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v)
{
	switch (index) {
	case 0: return plugin_example_rvo(A, N, c, v);
	}
	return 0;
}

}  // namespace umans
