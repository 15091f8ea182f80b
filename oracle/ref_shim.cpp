// Test-infrastructure shim over the UMANS reference engine (the oracle).
//
// This file is compiled together with the reference's own Engine sources by
// oracle/build_ref.sh into oracle/_ref/libumans_ref.so.  It is used only by
// tests, by the golden-fixture generator and by the CPU-baseline leg of
// bench.py; nothing in the product links it.
//
// It exposes the reference state through the reference's public accessors:
//   CrowdSimulator::FromConfigFile   (src/Engine/core/crowdSimulator.cpp:516)
//   CrowdSimulator::RunSimulationSteps (src/Engine/core/crowdSimulator.cpp:77)
//   WorldBase::GetAgents             (src/Engine/core/worldBase.h)
//   Agent::getNeighbors              (src/Engine/core/agent.h)
//   PhantomAgent::GetDistanceSquared (src/Engine/core/worldBase.h:56-77)
#include <core/crowdSimulator.h>
#include <core/worldBase.h>
#include <core/agent.h>
#include <chrono>

extern "C" {

void* uref_load(const char* path)
{
	return CrowdSimulator::FromConfigFile(path);
}

void uref_free(void* h)
{
	delete static_cast<CrowdSimulator*>(h);
}

int uref_num_agents(void* h)
{
	return (int)static_cast<CrowdSimulator*>(h)->GetWorld()->GetAgents().size();
}

double uref_time(void* h)
{
	return static_cast<CrowdSimulator*>(h)->GetWorld()->GetCurrentTime();
}

float uref_dt(void* h)
{
	return static_cast<CrowdSimulator*>(h)->GetWorld()->GetDeltaTime();
}

void uref_set_threads(void* h, int n)
{
	static_cast<CrowdSimulator*>(h)->GetWorld()->SetNumberOfThreads(n);
}

// Runs n steps and returns the wall time in seconds spent inside
// RunSimulationSteps (XML loading and output are outside the timed region).
double uref_step(void* h, int n)
{
	auto t0 = std::chrono::steady_clock::now();
	static_cast<CrowdSimulator*>(h)->RunSimulationSteps(n);
	auto t1 = std::chrono::steady_clock::now();
	return std::chrono::duration<double>(t1 - t0).count();
}

// Per-agent state in list order.  Any pointer may be null.
void uref_state(void* h, long long* ids, float* pos, float* vel, float* prefvel,
                float* viewdir, float* goal)
{
	const auto& agents = static_cast<CrowdSimulator*>(h)->GetWorld()->GetAgents();
	for (size_t i = 0; i < agents.size(); ++i)
	{
		const Agent* a = agents[i];
		if (ids) ids[i] = (long long)a->getID();
		if (pos) { pos[2 * i] = a->getPosition().x; pos[2 * i + 1] = a->getPosition().y; }
		if (vel) { vel[2 * i] = a->getVelocity().x; vel[2 * i + 1] = a->getVelocity().y; }
		if (prefvel) { prefvel[2 * i] = a->getPreferredVelocity().x; prefvel[2 * i + 1] = a->getPreferredVelocity().y; }
		if (viewdir) { viewdir[2 * i] = a->getViewingDirection().x; viewdir[2 * i + 1] = a->getViewingDirection().y; }
		if (goal) { goal[2 * i] = a->getGoal().x; goal[2 * i + 1] = a->getGoal().y; }
	}
}

// Neighbour list that agent `idx` used in the most recent step, in the
// reference's order: neighbour id, float distSqr and the (possibly
// wrap-displaced) neighbour position.  Returns the list length; at most
// `cap` entries are written.
int uref_neighbors(void* h, int idx, long long* ids, float* dist2, float* px, float* py, int cap)
{
	const auto& agents = static_cast<CrowdSimulator*>(h)->GetWorld()->GetAgents();
	const auto& nb = agents[idx]->getNeighbors().first;
	int n = (int)nb.size();
	for (int k = 0; k < n && k < cap; ++k)
	{
		ids[k] = (long long)nb[k].realAgent->getID();
		dist2[k] = nb[k].GetDistanceSquared();
		px[k] = nb[k].GetPosition().x;
		py[k] = nb[k].GetPosition().y;
	}
	return n;
}

}
