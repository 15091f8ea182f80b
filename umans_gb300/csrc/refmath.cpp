// Host side of the reference-exact exponential (refmath.hpp): builds the
// table of arguments where the C library's expf differs from ff_expf_core,
// caches it on disk, and uploads it once per device.
#include "refmath.hpp"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <sys/stat.h>

#include <cuda_runtime.h>
#if defined(__GLIBC__)
#include <gnu/libc-version.h>
#endif

namespace umans {

namespace {

struct HostTable {
	std::vector<uint2> slots;
	uint32_t mask = 0;
	int shift = 32;
	size_t count = 0;
	int fast = 0;
	float band = 0.0f;
};

std::mutex g_mutex;
HostTable* g_host = nullptr;
std::map<int, uint2*> g_dev;   // device ordinal -> slots

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

std::string cache_path()
{
	std::string dir;
	if (const char* d = std::getenv("UMANS_CACHE_DIR")) dir = d;
	else if (const char* h = std::getenv("HOME")) dir = std::string(h) + "/.cache/umans_gb300";
	else dir = "/tmp/umans_gb300";
	std::string libc = "unknown";
#if defined(__GLIBC__)
	libc = gnu_get_libc_version();
#endif
#if defined(__aarch64__)
	const char* arch = "aarch64";
#elif defined(__x86_64__)
	const char* arch = "x86_64";
#else
	const char* arch = "other";
#endif
	return dir + "/expf_exceptions_v1_" + arch + "_glibc" + libc + ".bin";
}

void mkdirs(const std::string& path)
{
	for (size_t p = path.find('/', 1); p != std::string::npos; p = path.find('/', p + 1))
		::mkdir(path.substr(0, p).c_str(), 0755);
}

std::vector<uint2> enumerate_exceptions()
{
	const uint32_t first = 0x80000000u;          // -0.0f
	const uint32_t last = fbits(FF_EXP_LO);       // -87.0f (most negative)
	unsigned nt = std::max(1u, std::thread::hardware_concurrency());
	std::vector<std::vector<uint2>> part(nt);
	std::vector<std::thread> th;
	const uint64_t total = (uint64_t)last - first + 1;
	for (unsigned t = 0; t < nt; ++t) {
		th.emplace_back([&, t]() {
			const uint64_t a = first + total * t / nt, b = first + total * (t + 1) / nt;
			auto& out = part[t];
			for (uint64_t u = a; u < b; ++u) {
				const float x = bitsf((uint32_t)u);
				const float mine = ff_expf_core(x);
				const float libc = expf(x);
				if (fbits(mine) != fbits(libc)) out.push_back(make_uint2((uint32_t)u, fbits(libc)));
			}
		});
	}
	for (auto& x : th) x.join();
	std::vector<uint2> all;
	for (auto& p : part) all.insert(all.end(), p.begin(), p.end());
	return all;
}

bool load_cache(const std::string& path, std::vector<uint2>& exc)
{
	FILE* f = std::fopen(path.c_str(), "rb");
	if (!f) return false;
	uint64_t n = 0;
	bool ok = std::fread(&n, 8, 1, f) == 1 && n < (1ull << 31);
	if (ok) {
		exc.resize(n);
		ok = n == 0 || std::fread(exc.data(), sizeof(uint2), n, f) == n;
	}
	std::fclose(f);
	return ok;
}

void save_cache(const std::string& path, const std::vector<uint2>& exc)
{
	mkdirs(path);
	std::string tmp = path + ".tmp" + std::to_string((unsigned long)std::hash<std::thread::id>()(std::this_thread::get_id()));
	FILE* f = std::fopen(tmp.c_str(), "wb");
	if (!f) return;
	uint64_t n = exc.size();
	bool ok = std::fwrite(&n, 8, 1, f) == 1 && (n == 0 || std::fwrite(exc.data(), sizeof(uint2), n, f) == n);
	std::fclose(f);
	if (ok) std::rename(tmp.c_str(), path.c_str());
	else std::remove(tmp.c_str());
}

HostTable* build_host_table()
{
	std::vector<uint2> exc;
	const std::string path = cache_path();
	if (!load_cache(path, exc)) {
		exc = enumerate_exceptions();
		save_cache(path, exc);
	}
	HostTable* T = new HostTable();
	uint32_t size = 1024;
	int lg = 10;
	while (size < 2 * exc.size() + 1) { size <<= 1; ++lg; }
	T->slots.assign(size, make_uint2(0, 0));
	T->mask = size - 1;
	T->shift = 32 - lg;
	for (const uint2& e : exc) {
		uint32_t h = ff_hash(e.x, T->shift);
		while (T->slots[h].x != 0) h = (h + 1) & T->mask;
		T->slots[h] = e;
	}
	T->count = exc.size();
	// the device may skip the table lookup away from rounding midpoints only
	// if every exception is a near-midpoint argument
	// (and the device's short evaluation answers only farther than `band`
	// from a midpoint, the largest distance of an exception)
	bool all_near = true;
	for (const uint2& e : exc) {
		bool near = false;
		float dist = 0.0f;
		ff_expf_core(bitsf(e.x), &near, &dist);
		all_near = all_near && near;
		T->band = std::max(T->band, dist);
	}
	T->fast = all_near ? 1 : 0;
	return T;
}

}  // namespace

float ref_expf_host(float x)
{
	// same decision as the device: table-backed inside the domain
	if (!(x >= FF_EXP_LO && x <= 0.0f)) return (float)std::exp((double)x);
	const float y = ff_expf_core(x);
	return y;
}

// Returns the device table (built on first use, shared by all simulations).
bool exp_exceptions_for_device(ExpExceptions* out, size_t* count, std::string& err)
{
	std::lock_guard<std::mutex> lk(g_mutex);
	if (!g_host) g_host = build_host_table();
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) { err = "cudaGetDevice failed"; return false; }
	auto it = g_dev.find(dev);
	if (it == g_dev.end()) {
		uint2* d = nullptr;
		if (cudaMalloc(&d, sizeof(uint2) * g_host->slots.size()) != cudaSuccess) { err = "cudaMalloc (exp table)"; return false; }
		if (cudaMemcpy(d, g_host->slots.data(), sizeof(uint2) * g_host->slots.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
			err = "cudaMemcpy (exp table)";
			return false;
		}
		it = g_dev.emplace(dev, d).first;
	}
	out->slots = it->second;
	out->mask = g_host->mask;
	out->shift = g_host->shift;
	out->fast = g_host->fast;
	out->band = g_host->band;
	if (count) *count = g_host->count;
	return true;
}

// ---------------------------------------------------------------------------
// sine and cosine (refmath.hpp: ff_sincos_core, ref_sincosf)

namespace {

struct ScHost {
	std::vector<uint2> sin_slots, cos_slots;
	uint32_t sin_mask = 0, cos_mask = 0;
	int sin_shift = 32, cos_shift = 32;
	float sin_near = 4.0f, cos_near = 4.0f;
	int sym = 1;
	size_t count = 0;
};

ScHost* g_sc_host = nullptr;
std::map<int, std::pair<uint2*, uint2*>> g_sc_dev;

std::string sc_cache_path()
{
	const std::string p = cache_path();   // .../expf_exceptions_v1_<arch>_glibc<ver>.bin
	const size_t slash = p.rfind('/');
	return p.substr(0, slash + 1) + "sincos_exceptions_v1" + p.substr(p.rfind("_v1_") + 3);
}

struct ScLists {
	std::vector<uint2> sin_exc, cos_exc;   // (argument bits, C library bits), both signs
	bool sym = true;                       // the C library is odd / even on the domain
};

ScLists sc_enumerate()
{
	const uint32_t last = fbits(SC_LIMIT);
	unsigned nt = std::max(1u, std::thread::hardware_concurrency());
	std::vector<ScLists> part(nt);
	std::vector<std::thread> th;
	const uint64_t total = (uint64_t)last + 1;
	for (unsigned t = 0; t < nt; ++t) {
		th.emplace_back([&, t]() {
			const uint64_t a = total * t / nt, b = total * (t + 1) / nt;
			ScLists& out = part[t];
			for (uint64_t u = a; u < b; ++u) {
				const float xp = bitsf((uint32_t)u);
				const float sp = sinf(xp), cp = cosf(xp);
				for (int sign = 0; sign < 2; ++sign) {
					const float x = sign ? -xp : xp;
					const float ls = sign ? sinf(x) : sp, lc = sign ? cosf(x) : cp;
					if (sign && (fbits(ls) != fbits(-sp) || fbits(lc) != fbits(cp))) out.sym = false;
					float ms, mc, rs, rc;
					ff_sincos_core(x, &ms, &mc, &rs, &rc);
					if (fbits(ms) != fbits(ls)) out.sin_exc.push_back(make_uint2(fbits(x), fbits(ls)));
					if (fbits(mc) != fbits(lc)) out.cos_exc.push_back(make_uint2(fbits(x), fbits(lc)));
				}
			}
		});
	}
	for (auto& x : th) x.join();
	ScLists all;
	for (auto& p : part) {
		all.sin_exc.insert(all.sin_exc.end(), p.sin_exc.begin(), p.sin_exc.end());
		all.cos_exc.insert(all.cos_exc.end(), p.cos_exc.begin(), p.cos_exc.end());
		all.sym = all.sym && p.sym;
	}
	return all;
}

bool sc_load_cache(const std::string& path, ScLists& L)
{
	FILE* f = std::fopen(path.c_str(), "rb");
	if (!f) return false;
	uint64_t h[3] = { 0, 0, 0 };
	bool ok = std::fread(h, 8, 3, f) == 3 && h[1] < (1ull << 31) && h[2] < (1ull << 31);
	if (ok) {
		L.sym = h[0] != 0;
		L.sin_exc.resize(h[1]);
		L.cos_exc.resize(h[2]);
		ok = (h[1] == 0 || std::fread(L.sin_exc.data(), sizeof(uint2), h[1], f) == h[1]) &&
		     (h[2] == 0 || std::fread(L.cos_exc.data(), sizeof(uint2), h[2], f) == h[2]);
	}
	std::fclose(f);
	return ok;
}

void sc_save_cache(const std::string& path, const ScLists& L)
{
	mkdirs(path);
	std::string tmp = path + ".tmp" + std::to_string((unsigned long)std::hash<std::thread::id>()(std::this_thread::get_id()));
	FILE* f = std::fopen(tmp.c_str(), "wb");
	if (!f) return;
	const uint64_t h[3] = { L.sym ? 1ull : 0ull, L.sin_exc.size(), L.cos_exc.size() };
	bool ok = std::fwrite(h, 8, 3, f) == 3 &&
	          (h[1] == 0 || std::fwrite(L.sin_exc.data(), sizeof(uint2), h[1], f) == h[1]) &&
	          (h[2] == 0 || std::fwrite(L.cos_exc.data(), sizeof(uint2), h[2], f) == h[2]);
	std::fclose(f);
	if (ok) std::rename(tmp.c_str(), path.c_str());
	else std::remove(tmp.c_str());
}

// hash table of the exceptions (positive keys only when the library is
// symmetric) and the smallest midpoint ratio among them
void sc_table(const std::vector<uint2>& exc, bool sym, bool want_sin, std::vector<uint2>& slots, uint32_t* mask,
              int* shift, float* near)
{
	std::vector<uint2> keep;
	for (const uint2& e : exc)
		if (!sym || !(e.x & 0x80000000u)) keep.push_back(e);
	uint32_t size = 1024;
	int lg = 10;
	while (size < 2 * keep.size() + 1) { size <<= 1; ++lg; }
	slots.assign(size, make_uint2(0, 0));
	*mask = size - 1;
	*shift = 32 - lg;
	float lo = 4.0f;
	for (const uint2& e : keep) {
		uint32_t h = ff_hash(e.x, *shift);
		while (slots[h].x != 0) h = (h + 1) & *mask;
		slots[h] = e;
	}
	for (const uint2& e : exc) {   // both signs: the device tests the ratio of its own argument
		float s, c, rs, rc;
		ff_sincos_core(bitsf(e.x), &s, &c, &rs, &rc);
		const float q = want_sin ? sc_midpoint_ratio(s, rs) : sc_midpoint_ratio(c, rc);
		lo = std::min(lo, q);
	}
	*near = lo;
}

ScHost* sc_build_host()
{
	ScLists L;
	const std::string path = sc_cache_path();
	if (!sc_load_cache(path, L)) {
		L = sc_enumerate();
		sc_save_cache(path, L);
	}
	// symmetric keys need the negative exceptions to mirror the positive ones
	if (L.sym) {
		for (const std::vector<uint2>* v : { &L.sin_exc, &L.cos_exc }) {
			std::vector<uint32_t> pos, neg;
			for (const uint2& e : *v) (e.x & 0x80000000u ? neg : pos).push_back(e.x & 0x7fffffffu);
			std::sort(pos.begin(), pos.end());
			std::sort(neg.begin(), neg.end());
			if (pos != neg) L.sym = false;
		}
	}
	ScHost* T = new ScHost();
	T->sym = L.sym ? 1 : 0;
	sc_table(L.sin_exc, L.sym, true, T->sin_slots, &T->sin_mask, &T->sin_shift, &T->sin_near);
	sc_table(L.cos_exc, L.sym, false, T->cos_slots, &T->cos_mask, &T->cos_shift, &T->cos_near);
	T->count = L.sin_exc.size() + L.cos_exc.size();
	return T;
}

bool upload(const std::vector<uint2>& v, uint2** d, std::string& err)
{
	if (cudaMalloc(d, sizeof(uint2) * v.size()) != cudaSuccess) { err = "cudaMalloc (sincos table)"; return false; }
	if (cudaMemcpy(*d, v.data(), sizeof(uint2) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
		err = "cudaMemcpy (sincos table)";
		return false;
	}
	return true;
}

}  // namespace

bool sincos_exceptions_for_device(SinCosExceptions* out, size_t* count, std::string& err)
{
	std::lock_guard<std::mutex> lk(g_mutex);
	if (!g_sc_host) g_sc_host = sc_build_host();
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) { err = "cudaGetDevice failed"; return false; }
	auto it = g_sc_dev.find(dev);
	if (it == g_sc_dev.end()) {
		uint2 *ds = nullptr, *dc = nullptr;
		if (!upload(g_sc_host->sin_slots, &ds, err) || !upload(g_sc_host->cos_slots, &dc, err)) return false;
		it = g_sc_dev.emplace(dev, std::make_pair(ds, dc)).first;
	}
	out->sin_slots = it->second.first;
	out->cos_slots = it->second.second;
	out->sin_mask = g_sc_host->sin_mask;
	out->cos_mask = g_sc_host->cos_mask;
	out->sin_shift = g_sc_host->sin_shift;
	out->cos_shift = g_sc_host->cos_shift;
	out->sin_near = g_sc_host->sin_near;
	out->cos_near = g_sc_host->cos_near;
	out->sym = g_sc_host->sym;
	if (count) *count = g_sc_host->count;
	return true;
}

}  // namespace umans
