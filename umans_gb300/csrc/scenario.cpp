#include "scenario.hpp"
#include "plugins.hpp"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <set>

#include "xml.hpp"

namespace umans {

static const double REF_PI = 3.1415926535897;   // vector2D.h:27

static const char* KIND_NAMES[K_NUM_KINDS] = {
	"ORCA", "RVO", "SocialForcesAvoidance", "PowerLaw", "GoalReachingForce", "Karamouzas",
	"Moussaid", "Paris", "VanToll", "TtcaDca", "FOEAvoidance", "PLEdestrians", "RandomFunction", "Generic"};

const char* cost_kind_name(int kind)
{
	if (kind >= 0 && kind < K_NUM_KINDS) return KIND_NAMES[kind];
	if (kind >= K_PLUGIN0 && kind < K_PLUGIN0 + kNumPlugins) return kPlugins[kind - K_PLUGIN0].name;
	return "?";
}

int cost_function_count() { return K_NUM_KINDS + kNumPlugins; }

const char* cost_function_name(int index)
{
	if (index < 0 || index >= cost_function_count()) return nullptr;
	return cost_kind_name(index < K_NUM_KINDS ? index : K_PLUGIN0 + (index - K_NUM_KINDS));
}

int cost_kind_from_name(const std::string& name)
{
	for (int k = 0; k < K_NUM_KINDS; ++k)
		if (name == KIND_NAMES[k]) return k;
	for (int k = 0; k < kNumPlugins; ++k)   // costFunctionFactory.cpp:41-61: registered plugins by name
		if (name == kPlugins[k].name) return K_PLUGIN0 + k;
	return -1;
}

void cost_defaults(int kind, CostDesc& c)
{
	std::memset(&c, 0, sizeof(c));
	c.kind = kind;
	c.coeff = 1;
	c.range = 5.0f;   // CostFunction::range_ (costFunction.h:128)
	switch (kind) {
	case K_ORCA: c.p[0] = 5; break;                                   // ORCA.h:54
	case K_RVO: c.p[0] = 1; break;                                    // RVO.h:53
	case K_SOCIALFORCES:                                              // SocialForcesAvoidance.h:57-61
		c.p[0] = 1; c.p[1] = 2.1f; c.p[2] = 0.3f; c.p[3] = 10; c.p[4] = 0.2f; c.p[5] = 1; break;
	case K_POWERLAW: c.p[0] = 1.5f; c.p[1] = 3; c.p[5] = 1; break;    // PowerLaw.h:57-58
	case K_GOALREACHING: c.p[5] = 1; c.range = 0; break;              // GoalReachingForce.h:38
	case K_KARAMOUZAS: c.p[0] = 5; c.p[1] = 0.5f; c.p[2] = 1; c.p[3] = 1; c.p[4] = 8; break;
	case K_MOUSSAID: c.p[0] = 8; break;
	case K_PARIS: c.p[0] = 0.5f; c.p[1] = 0; c.p[2] = 8; break;
	case K_VANTOLL: c.p[0] = 8; break;
	case K_TTCADCA: c.p[0] = 2; c.p[1] = 2; c.p[2] = 1; c.p[3] = 0.3f; break;
	case K_PLEDESTRIANS: c.p[0] = 2.23f; c.p[1] = 1.26f; c.p[2] = 0.5f; c.p[3] = 3; break;
	case K_RANDOM: c.range = 0; break;                                 // RandomFunction.h: range_ = 0
	default:
		if (kind >= K_PLUGIN0 && kind < K_PLUGIN0 + kNumPlugins) {
			const PluginInfo& pl = kPlugins[kind - K_PLUGIN0];
			for (int k = 0; k < pl.nparams; ++k) c.p[pl.params[k].slot] = pl.params[k].dflt;
			if (pl.range >= 0) c.range = pl.range;
		}
		break;
	}
}

// parseParameters of each plugin (CostFunctions/*.cpp); ForceBasedFunction
// adds agentMass (ForceBasedFunction.cpp:42-46).
static void parse_cost_params(const XmlElement* e, CostDesc& c)
{
	e->query_float("range", &c.range);
	auto rd = [&](const char* k, int slot) { e->query_float(k, &c.p[slot]); };
	switch (c.kind) {
	case K_ORCA: rd("timeHorizon", 0); break;
	case K_RVO: rd("w", 0); break;
	case K_SOCIALFORCES:
		rd("agentMass", 5); rd("dt", 0); rd("V0", 1); rd("sigma", 2);
		rd("U0", 1);   // sic: SocialForcesAvoidance.cpp:148 reads "U0" into V0
		rd("R", 4);
		break;
	case K_POWERLAW: rd("agentMass", 5); rd("k", 0); rd("tau0", 1); break;
	case K_GOALREACHING: rd("agentMass", 5); break;
	case K_KARAMOUZAS: rd("alpha", 0); rd("beta", 1); rd("gamma", 2); rd("delta", 3); rd("t_max", 4); break;
	case K_MOUSSAID: rd("d_max", 0); break;
	case K_PARIS: rd("w_a", 0); rd("w_b", 1); rd("t_max", 2); break;
	case K_VANTOLL: rd("max_distance", 0); break;
	case K_TTCADCA: rd("sigmaAngle_goal", 0); rd("sigmaSpeed_goal", 1); rd("sigmaTtca", 2); rd("sigmaDca", 3); break;
	case K_PLEDESTRIANS: rd("w_a", 0); rd("w_b", 1); rd("t_min", 2); rd("t_max", 3); break;
	default:
		if (c.kind >= K_PLUGIN0 && c.kind < K_PLUGIN0 + kNumPlugins) {
			const PluginInfo& pl = kPlugins[c.kind - K_PLUGIN0];
			for (int k = 0; k < pl.nparams; ++k) rd(pl.params[k].attr, pl.params[k].slot);
		}
		break;
	}
}

static std::string folder_of(const std::string& f)
{
	auto p = f.find_last_of('/');
	return p == std::string::npos ? std::string() : f.substr(0, p + 1);
}

namespace {
struct Loader {
	Scenario& s;
	std::string& err;
	std::set<int> active_ids;

	bool policy(const XmlElement* pe)
	{   // FromConfigFile_loadSinglePolicy: crowdSimulator.cpp:327-422
		int pid = 0;
		pe->query_int("id", &pid);
		const char* m = pe->attr("OptimizationMethod");
		std::string ms = m ? m : "";
		PolicyDesc p;
		std::memset(&p, 0, sizeof(p));
		if (ms == "gradient") p.method = M_GRADIENT;
		else if (ms == "sampling") p.method = M_SAMPLING;
		else if (ms == "global") p.method = M_GLOBAL;
		else { err = "Policy " + std::to_string(pid) + ": optimization method invalid"; return false; }
		// SamplingParameters defaults: policy.h:59-67
		p.s_type = 0; p.s_base = 0; p.s_dir = 1; p.s_radius = 0;
		p.s_angle = 180; p.speed_samples = 4; p.angle_samples = 11; p.random_samples = 100; p.include_base = 0;
		if (p.method == M_SAMPLING) {
			pe->query_float("SamplingAngle", &p.s_angle);
			pe->query_int("SpeedSamples", &p.speed_samples);
			pe->query_int("AngleSamples", &p.angle_samples);
			pe->query_int("RandomSamples", &p.random_samples);
			bool b;
			if (pe->query_bool("IncludeBaseAsSample", &b)) p.include_base = b ? 1 : 0;
			std::string v;
			if (const char* a = pe->attr("SamplingType")) {
				v = a;
				if (v == "regular") p.s_type = 0; else if (v == "random") p.s_type = 1;
				else s.warnings.push_back("Policy " + std::to_string(pid) + ": sampling type invalid, using default (regular)");
			}
			if (const char* a = pe->attr("SamplingBase")) {
				v = a;
				if (v == "zero") p.s_base = 0; else if (v == "current velocity") p.s_base = 1;
				else s.warnings.push_back("Policy " + std::to_string(pid) + ": sampling base invalid, using default (zero)");
			}
			if (const char* a = pe->attr("SamplingBaseDirection")) {
				v = a;
				if (v == "unit") p.s_dir = 0; else if (v == "current velocity") p.s_dir = 1;
				else if (v == "preferred velocity") p.s_dir = 2;
				else s.warnings.push_back("Policy " + std::to_string(pid) + ": sampling base direction invalid, using default");
			}
			if (const char* a = pe->attr("SamplingRadius")) {
				v = a;
				if (v == "preferred speed") p.s_radius = 0; else if (v == "maximum speed") p.s_radius = 1;
				else if (v == "maximum acceleration") p.s_radius = 2;
				else s.warnings.push_back("Policy " + std::to_string(pid) + ": sampling radius type invalid, using default");
			}
		}
		p.relax_time = 0;
		pe->query_float("RelaxationTime", &p.relax_time);
		p.contact_scale = 5000;   // policy.h:125
		pe->query_float("ContactForceScale", &p.contact_scale);
		// cost functions: first "costfunction" child, then every following sibling
		const XmlElement* fe = pe->first_child("costfunction");
		while (fe) {
			const char* nm = fe->attr("name");
			int kind = cost_kind_from_name(nm ? nm : "");
			if (kind == -2) { err = std::string("cost function ") + nm + " is not supported by this engine"; return false; }
			if (kind >= 0) {
				if (p.ncost == MAX_COSTS) { err = "more than 4 cost functions in a policy"; return false; }
				CostDesc& c = p.cost[p.ncost];
				cost_defaults(kind, c);
				fe->query_float("coeff", &c.coeff);   // Policy::AddCostFunction: policy.cpp:143-149
				parse_cost_params(fe, c);
				p.ncost++;
			} else {
				s.warnings.push_back("Policy " + std::to_string(pid) + ": unknown cost function " + std::string(nm ? nm : "(null)") + " ignored");
			}
			fe = pe->next_sibling(fe);
		}
		if (p.ncost == 0) { err = "Policy " + std::to_string(pid) + " needs at least one cost function element"; return false; }
		for (int id : s.policy_ids)
			if (id == pid) { err = "policy id " + std::to_string(pid) + " is already taken"; return false; }
		p.max_angle = (float)(p.s_angle / 360.0 * REF_PI);
		float r = 0;
		for (int c = 0; c < p.ncost; ++c) r = std::max(r, p.cost[c].range);
		p.range = r;
		s.policies.push_back(p);
		s.policy_ids.push_back(pid);
		return true;
	}

	bool obstacle(const XmlElement* oe)
	{   // FromConfigFile_loadSingleObstacle: crowdSimulator.cpp:496-514, then
		// WorldBase::AddObstacle (worldBase.cpp:239-242): the polygon's edges
		std::vector<float2> pts;
		for (const XmlElement* pe = oe->first_child("Point"); pe; pe = oe->next_sibling(pe, "Point")) {
			float x = 0, y = 0;
			pe->query_float("x", &x);
			pe->query_float("y", &y);
			pts.push_back(float2{ x, y });
		}
		const size_t n = pts.size();
		for (size_t i = 0; i < n; ++i) {
			const float2 a = pts[i], b = pts[(i + 1) % n];
			s.edges.push_back(float4{ a.x, a.y, b.x, b.y });
		}
		return true;
	}

	bool agent(const XmlElement* ae)
	{   // FromConfigFile_loadSingleAgent: crowdSimulator.cpp:424-494
		int want = -1;
		ae->query_int("id", &want);
		AgentInit a;
		a.radius = 0.24f; a.pref_speed = 1.4f; a.max_speed = 1.8f; a.max_accel = 5.0f;   // agent.h:44-53
		a.remove_at_goal = false;
		ae->query_float("rad", &a.radius);
		ae->query_float("pref_speed", &a.pref_speed);
		ae->query_float("max_speed", &a.max_speed);
		ae->query_float("max_acceleration", &a.max_accel);
		ae->query_bool("remove_at_goal", &a.remove_at_goal);
		const XmlElement* pos = ae->first_child("pos");
		if (!pos) { err = "Agent needs a position element"; return false; }
		float x = 0, y = 0;
		pos->query_float("x", &x);
		pos->query_float("y", &y);
		const XmlElement* pol = ae->first_child("Policy");
		if (!pol) { err = "Agent needs a policy element"; return false; }
		int ppid = 0;
		pol->query_int("id", &ppid);
		int pidx = -1;
		for (size_t k = 0; k < s.policy_ids.size(); ++k)
			if (s.policy_ids[k] == ppid) pidx = (int)k;
		if (pidx < 0) { err = "The policy with id " + std::to_string(ppid) + " doesn't exist"; return false; }
		a.policy = pidx;
		a.start_time = 0;
		ae->query_float("start_time", &a.start_time);
		// WorldBase::AddAgent id rule: worldBase.cpp:161-186
		int id;
		if (want >= 0 && !active_ids.count(want)) id = want;
		else id = s.next_unused_id;
		if (id >= s.next_unused_id) s.next_unused_id = id + 1;
		a.id = id;
		if (a.start_time <= 0) active_ids.insert(id);
		a.x = x; a.y = y;
		a.gx = x; a.gy = y;
		if (const XmlElement* g = ae->first_child("goal")) {
			g->query_float("x", &x);
			g->query_float("y", &y);
			a.gx = x; a.gy = y;
		} else {
			s.warnings.push_back("agent has no goal element and will not move");
		}
		s.agents.push_back(a);
		return true;
	}

	// ...ExternallyOrNot: crowdSimulator.cpp:210-274; blocks: :276-325
	template <class F>
	bool block(const XmlElement* b, const std::string& folder, const char* blockName, const char* itemName, F each,
	           XmlDocument& ext)
	{
		if (const char* f = b->attr("file")) {
			if (!ext.load_file(folder + f)) { err = std::string("Could not load or parse ") + blockName + " XML file at " + folder + f; return false; }
			b = ext.root.first_child(blockName);
			if (!b) { err = std::string("no ") + blockName + " element in " + folder + f; return false; }
		}
		const XmlElement* e = b->first_child();
		while (e) {
			if (!each(e)) return false;
			e = b->next_sibling(e, itemName);
		}
		return true;
	}
};
}  // namespace

bool load_scenario(const std::string& path, Scenario& s, std::string& err)
{
	s = Scenario();
	s.end_time = FLT_MAX;
	XmlDocument doc;
	if (!doc.load_file(path)) { err = "Could not load or parse XML file at " + path + ": " + doc.error; return false; }
	const std::string folder = folder_of(path);
	if (const XmlElement* cp = doc.root.first_child("configPath")) {
		const char* p = cp->attr("path");
		return load_scenario(folder + (p ? p : ""), s, err);
	}
	const XmlElement* sim = doc.root.first_child("Simulation");
	if (!sim) { err = "No main Simulation element in the XML file"; return false; }
	const XmlElement* world = sim->first_child("World");
	if (!world) { err = "No World element in the XML file"; return false; }
	// FromConfigFile_loadWorld: crowdSimulator.cpp:167-208
	const char* wt = world->attr("type");
	std::string wts = wt ? wt : "";
	if (wts == "Toric") {
		float w = -1, h = -1;
		world->query_float("width", &w);
		world->query_float("height", &h);
		if (!(w > 0 && h > 0)) { err = "No valid size specified for the toric world"; return false; }
		s.world = W_TORIC; s.width = w; s.height = h;
	} else {
		if (wts != "Infinite") s.warnings.push_back("no valid world type; using Infinite");
		s.world = W_INFINITE;
	}
	float dt = -1;
	sim->query_float("delta_time", &dt);
	if (dt <= 0) { err = "No valid value for delta_time found in the XML file"; return false; }
	s.dt = dt;
	sim->query_float("end_time", &s.end_time);

	Loader L{s, err, {}};
	XmlDocument ext1, ext2;
	if (const XmlElement* pb = sim->first_child("Policies")) {
		if (!L.block(pb, folder, "Policies", "Policy", [&](const XmlElement* e) { return L.policy(e); }, ext1)) return false;
	}
	if (s.policies.empty()) { err = "Failed to load any policies for the simulation"; return false; }
	if (const XmlElement* ab = sim->first_child("Agents")) {
		if (!L.block(ab, folder, "Agents", "Agent", [&](const XmlElement* e) { return L.agent(e); }, ext2)) return false;
	}
	// FromConfigFile: obstacles after the agents (crowdSimulator.cpp:633-645)
	XmlDocument ext3;
	if (const XmlElement* ob = world->first_child("Obstacles")) {
		if (!L.block(ob, folder, "Obstacles", "Obstacle", [&](const XmlElement* e) { return L.obstacle(e); }, ext3))
			return false;
	}
	return true;
}

}  // namespace umans
