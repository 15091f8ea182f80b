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
	bool all_near = true;
	for (const uint2& e : exc) {
		bool near = false;
		ff_expf_core(bitsf(e.x), &near);
		all_near = all_near && near;
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
	if (count) *count = g_host->count;
	return true;
}

}  // namespace umans
