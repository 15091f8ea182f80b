// Reference-exact float exponential for the device.
//
// The reference evaluates exp(float) with the host C library's expf
// (SocialForcesAvoidance.cpp:98, PowerLaw.cpp:62, FOEAvoidance.cpp:82), and
// the crowd dynamics amplify a last-bit difference into centimetres within a
// few dozen steps.  The host expf is not correctly rounded in every case, so
// no independent implementation equals it bit for bit.  Instead:
//
//  * ff_expf() below is a table-driven exponential (Tang's method: x =
//    k ln2/64 + r, e^x = 2^(k/64) e^r) evaluated in float-float arithmetic
//    (~2^-45 relative before the final rounding).  It uses only IEEE float
//    +,-,* (Veltkamp/Dekker exact products, no FMA), so it gives identical
//    results when compiled for the host and for the GPU;
//  * at start-up the host runs ff_expf and the C library's expf on every
//    float in [-87, 0] and records the inputs where they differ (the C
//    library's own misroundings plus ours, ~1e-3 of the inputs) in an
//    open-addressing table;
//  * the device evaluates ff_expf and then looks its argument up in that
//    table, which returns exactly the host expf's value.
// Outside [-87, 0] (never reached by the force models, whose arguments are
// -b/sigma, -tau/tau0 and -|dx|/sigma) the value is (float)exp((double)x).
#pragma once
#include <cstdint>
#include <cmath>

#include <string>

#include <vector_types.h>

#if defined(__CUDACC__)
#define RM_HD __host__ __device__ __forceinline__
#else
#define RM_HD inline
#endif

namespace umans {

struct FF { float h, l; };

RM_HD FF ff_two_sum(float a, float b)
{
	const float s = a + b;
	const float bb = s - a;
	const float e = (a - (s - bb)) + (b - bb);
	return FF{ s, e };
}
RM_HD FF ff_fast_two_sum(float a, float b)   // |a| >= |b|
{
	const float s = a + b;
	return FF{ s, b - (s - a) };
}
RM_HD void ff_split(float a, float* hi, float* lo)   // Veltkamp, 12 + 12 bits
{
	const float c = 4097.0f * a;
	const float h = c - (c - a);
	*hi = h;
	*lo = a - h;
}
// exact product a*b = p + e (no overflow or underflow in the uses below):
// an FMA on the GPU, Dekker's product on the host; both give the same exact e
RM_HD FF ff_two_prod(float a, float b)
{
	const float p = a * b;
#if defined(__CUDA_ARCH__)
	return FF{ p, fmaf(a, b, -p) };
#else
	float ah, al, bh, bl;
	ff_split(a, &ah, &al);
	ff_split(b, &bh, &bl);
	const float e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
	return FF{ p, e };
#endif
}

RM_HD uint32_t rm_bits(float f)
{
#if defined(__CUDA_ARCH__)
	return __float_as_uint(f);
#else
	union { float f; uint32_t u; } c; c.f = f; return c.u;
#endif
}
RM_HD float rm_float(uint32_t u)
{
#if defined(__CUDA_ARCH__)
	return __uint_as_float(u);
#else
	union { uint32_t u; float f; } c; c.u = u; return c.f;
#endif
}

// 2^(j/64) = hi + lo (hi + lo within 2^-48 of the exact value); one copy
// for the host, one in device global memory
#if defined(__CUDACC__)
static __device__ const float FF_EXP2_TAB_D[64][2] = {
	{ 0x1.0000000000000p+0f, 0x0.0p+0f },
	{ 0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f },
	{ 0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f },
	{ 0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f },
	{ 0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f },
	{ 0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f },
	{ 0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f },
	{ 0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f },
	{ 0x1.172b840000000p+0f, -0x1.c157420000000p-27f },
	{ 0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f },
	{ 0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f },
	{ 0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f },
	{ 0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f },
	{ 0x1.26b4560000000p+0f, 0x1.789f380000000p-26f },
	{ 0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f },
	{ 0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f },
	{ 0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f },
	{ 0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f },
	{ 0x1.371a740000000p+0f, -0x1.18aac60000000p-25f },
	{ 0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f },
	{ 0x1.3dea640000000p+0f, 0x1.8246840000000p-25f },
	{ 0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f },
	{ 0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f },
	{ 0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f },
	{ 0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f },
	{ 0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f },
	{ 0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f },
	{ 0x1.56f4740000000p+0f, -0x1.295b040000000p-25f },
	{ 0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f },
	{ 0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f },
	{ 0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f },
	{ 0x1.6623880000000p+0f, 0x1.2a91120000000p-27f },
	{ 0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f },
	{ 0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f },
	{ 0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f },
	{ 0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f },
	{ 0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f },
	{ 0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f },
	{ 0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f },
	{ 0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f },
	{ 0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f },
	{ 0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f },
	{ 0x1.93737c0000000p+0f, -0x1.e647440000000p-25f },
	{ 0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f },
	{ 0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f },
	{ 0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f },
	{ 0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f },
	{ 0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f },
	{ 0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f },
	{ 0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f },
	{ 0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f },
	{ 0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f },
	{ 0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f },
	{ 0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f },
	{ 0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f },
	{ 0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f },
	{ 0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f },
	{ 0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f },
	{ 0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f },
	{ 0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f },
	{ 0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f },
	{ 0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f },
	{ 0x1.f507660000000p+0f, -0x1.246eb00000000p-26f },
	{ 0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f },
};
#endif
static const float FF_EXP2_TAB_H[64][2] = {
	{ 0x1.0000000000000p+0f, 0x0.0p+0f },
	{ 0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f },
	{ 0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f },
	{ 0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f },
	{ 0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f },
	{ 0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f },
	{ 0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f },
	{ 0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f },
	{ 0x1.172b840000000p+0f, -0x1.c157420000000p-27f },
	{ 0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f },
	{ 0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f },
	{ 0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f },
	{ 0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f },
	{ 0x1.26b4560000000p+0f, 0x1.789f380000000p-26f },
	{ 0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f },
	{ 0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f },
	{ 0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f },
	{ 0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f },
	{ 0x1.371a740000000p+0f, -0x1.18aac60000000p-25f },
	{ 0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f },
	{ 0x1.3dea640000000p+0f, 0x1.8246840000000p-25f },
	{ 0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f },
	{ 0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f },
	{ 0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f },
	{ 0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f },
	{ 0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f },
	{ 0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f },
	{ 0x1.56f4740000000p+0f, -0x1.295b040000000p-25f },
	{ 0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f },
	{ 0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f },
	{ 0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f },
	{ 0x1.6623880000000p+0f, 0x1.2a91120000000p-27f },
	{ 0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f },
	{ 0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f },
	{ 0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f },
	{ 0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f },
	{ 0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f },
	{ 0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f },
	{ 0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f },
	{ 0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f },
	{ 0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f },
	{ 0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f },
	{ 0x1.93737c0000000p+0f, -0x1.e647440000000p-25f },
	{ 0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f },
	{ 0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f },
	{ 0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f },
	{ 0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f },
	{ 0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f },
	{ 0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f },
	{ 0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f },
	{ 0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f },
	{ 0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f },
	{ 0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f },
	{ 0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f },
	{ 0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f },
	{ 0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f },
	{ 0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f },
	{ 0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f },
	{ 0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f },
	{ 0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f },
	{ 0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f },
	{ 0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f },
	{ 0x1.f507660000000p+0f, -0x1.246eb00000000p-26f },
	{ 0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f },
};

RM_HD float ff_exp2_tab(int j, int w)
{
#if defined(__CUDA_ARCH__)
	return FF_EXP2_TAB_D[j][w];
#else
	return FF_EXP2_TAB_H[j][w];
#endif
}

constexpr float FF_EXP_LO = -87.0f;

// e^x for x in [FF_EXP_LO, 0]; the caller checks the range.  *near is set
// when the unrounded value lies within 1/256 ulp of a rounding midpoint (the
// only place where the host library's expf, accurate to 0.502 ulp, and this
// function can disagree; the host verifies that against its full table).
RM_HD float ff_expf_core(float x, bool* near = nullptr)
{
	const float INV = 92.33248138427734f;      // 64 / ln 2
	const float L1 = 0x1.62cp-7f;              // ln2/64 = L1 + L2 + L3, L1 with 11 bits
	const float L2 = 0x1.217f7ep-18f;
	const float L3 = -0x1.c610cap-43f;
	const float kf = rintf(x * INV);
	const int k = (int)kf;
	const float t1 = x - kf * L1;              // kf*L1 exact; difference exact (Sterbenz)
	const FF q = ff_two_prod(kf, L2);
	const FF r0 = ff_two_sum(t1, -q.h);
	const float rl0 = (r0.l - q.l) - kf * L3;
	const FF r = ff_fast_two_sum(r0.h, rl0);
	const float h = r.h, l = r.l;
	// e^r - 1 = r + r^2/2 + r^3/6 + r^4/24 + r^5/120 + r^6/720
	const FF h2 = ff_two_prod(h, h);
	float tail = (1.0f / 6.0f) + h * ((1.0f / 24.0f) + h * ((1.0f / 120.0f) + h * (1.0f / 720.0f)));
	tail = tail * (h * h * h) + (h * h * l) * 0.5f;
	const FF a = ff_two_sum(h, h2.h * 0.5f);
	const float lo = a.l + (l + (h2.l * 0.5f + (h * l + tail)));
	const FF s = ff_fast_two_sum(1.0f, a.h);
	const float sl = s.l + lo;
	const int j = k & 63;
	const int kq = (k - j) / 64;               // floor(k / 64)
	const float Th = ff_exp2_tab(j, 0), Tl = ff_exp2_tab(j, 1);
	const FF m = ff_two_prod(Th, s.h);
	const float ml = m.l + (Th * sl + Tl * s.h);
	const float f = m.h + ml;
	if (near) {
		const float rl = ml - (f - m.h);
		const float half_ulp = rm_float((rm_bits(f) & 0x7f800000u) - (24u << 23));
		*near = !(fabsf(rl) < half_ulp * 0.99609375f);
	}
	// 2^kq, kq in [-126, 0]: normal, so the scaling is exact
	return f * rm_float((uint32_t)(kq + 127) << 23);
}

// open-addressing table of (argument bits, host expf bits); key 0 = empty
struct ExpExceptions {
	const uint2* slots;
	uint32_t mask;    // size - 1 (size a power of two)
	int shift;        // 32 - log2(size)
	int fast;         // 1 when every table entry is a near-midpoint argument
};

RM_HD uint32_t ff_hash(uint32_t bits, int shift) { return (bits * 0x9E3779B1u) >> shift; }

#if defined(__CUDACC__)
// The host C library's expf(x), exactly (see the header comment).
__device__ __forceinline__ float ref_expf(const ExpExceptions& T, float x)
{
	if (!(x >= FF_EXP_LO && x <= 0.0f)) return (float)exp((double)x);
	bool near;
	const float y = ff_expf_core(x, &near);
	if (T.fast && !near) return y;
	const uint32_t b = __float_as_uint(x);
	uint32_t h = ff_hash(b, T.shift);
	for (;;) {
		const uint2 e = __ldg(&T.slots[h]);
		if (e.x == 0) return y;   // empty slot (keys are never 0: +0.0 is not stored)
		if (e.x == b) return __uint_as_float(e.y);
		h = (h + 1) & T.mask;
	}
}
#endif

// host side (refmath.cpp): table shared by all simulations on a device
bool exp_exceptions_for_device(ExpExceptions* out, size_t* count, std::string& err);

}  // namespace umans
