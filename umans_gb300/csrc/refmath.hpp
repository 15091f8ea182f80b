// Reference-exact arithmetic shared by the host and the device:
//  * the host C library's expf (this header comment), sinf and cosf (the
//    section "Reference-exact float sine and cosine" below), reproduced bit
//    for bit on the device;
//  * the reference's double line intersection without FP64 in the common
//    case (getLineIntersection section);
//  * the double Gaussians of TtcaDca rounded to float (exp_gauss).
// Every part is float-float arithmetic with exact products (FMA on the
// device, Dekker on the host), so host and device compute the same bits, and
// falls back to the exact computation where its error bound cannot decide.
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
// *dist receives that distance from the midpoint in ulps of the result.
RM_HD float ff_expf_core(float x, bool* near = nullptr, float* dist = nullptr)
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
	if (near || dist) {
		const float rl = ml - (f - m.h);
		const float half_ulp = rm_float((rm_bits(f) & 0x7f800000u) - (24u << 23));
		if (near) *near = !(fabsf(rl) < half_ulp * 0.99609375f);
		if (dist) *dist = (half_ulp - fabsf(rl)) / (2.0f * half_ulp);
	}
	// 2^kq, kq in [-126, 0]: normal, so the scaling is exact
	return f * rm_float((uint32_t)(kq + 127) << 23);
}

// e^(xh + xl) for xh in [FF_EXP_LO, 0] and |xl| <= ulp(xh): the same
// reduction and series as ff_expf_core with the low part of the argument
// added to the reduced argument; returns the unrounded value hi + lo in
// [2^-1, 2^1] and the exact scale 2^kq (the result is (hi + lo) * scale).
RM_HD void ff_exp_ff(float xh, float xl, float* hi, float* lo, float* scale)
{
	const float INV = 92.33248138427734f;      // 64 / ln 2
	const float L1 = 0x1.62cp-7f;              // ln2/64 = L1 + L2 + L3, L1 with 11 bits
	const float L2 = 0x1.217f7ep-18f;
	const float L3 = -0x1.c610cap-43f;
	const float kf = rintf(xh * INV);
	const int k = (int)kf;
	const float t1 = xh - kf * L1;             // kf*L1 exact; difference exact (Sterbenz)
	const FF q = ff_two_prod(kf, L2);
	const FF r0 = ff_two_sum(t1, -q.h);
	const float rl0 = ((r0.l - q.l) - kf * L3) + xl;
	const FF r = ff_two_sum(r0.h, rl0);
	const float h = r.h, l = r.l;
	const FF h2 = ff_two_prod(h, h);
	float tail = (1.0f / 6.0f) + h * ((1.0f / 24.0f) + h * ((1.0f / 120.0f) + h * (1.0f / 720.0f)));
	tail = tail * (h * h * h) + (h * h * l) * 0.5f;
	const FF a = ff_two_sum(h, h2.h * 0.5f);
	const float lo0 = a.l + (l + (h2.l * 0.5f + (h * l + tail)));
	const FF s = ff_fast_two_sum(1.0f, a.h);
	const float sl = s.l + lo0;
	const int j = k & 63;
	const int kq = (k - j) / 64;               // floor(k / 64)
	const float Th = ff_exp2_tab(j, 0), Tl = ff_exp2_tab(j, 1);
	const FF m = ff_two_prod(Th, s.h);
	*hi = m.h;
	*lo = m.l + (Th * sl + Tl * s.h);
	*scale = rm_float((uint32_t)(kq + 127) << 23);   // kq in [-126, 0]
}

// open-addressing table of (argument bits, host expf bits); key 0 = empty
struct ExpExceptions {
	const uint2* slots;
	uint32_t mask;    // size - 1 (size a power of two)
	int shift;        // 32 - log2(size)
	int fast;         // 1 when every table entry is a near-midpoint argument
	float band;       // largest distance of an entry's value from its rounding midpoint, in ulps
};

RM_HD uint32_t ff_hash(uint32_t bits, int shift) { return (bits * 0x9E3779B1u) >> shift; }

#if defined(__CUDACC__)
// ln 2 / 64 = EXP_L1 + EXP_L2 (+ 1.4e-18); EXP_L1 is a multiple of 2^-30
constexpr float EXP_L1 = 0x1.62e43p-7f;
constexpr float EXP_L2 = -0x1.05c61p-35f;

// e^x for x in [FF_EXP_LO, 0] by a short FMA evaluation: Tang's table method
// (P. T. P. Tang, "Table-driven implementation of the exponential function
// in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989), x = k ln2/64 + r
// with r reduced in two parts (the first, fma(-k, EXP_L1, x), is exact: both
// terms are multiples of 2^-30 and |r| < 2^-7), e^r - 1 by a degree-4
// polynomial, and 2^(j/64) from the float-pair table; the unrounded value is
// within 2^-13 ulp of e^x.  Returns true with *out = e^x rounded to nearest
// when that rounding is decided and e^x lies farther than `band` + 2^-13 ulp
// from a rounding midpoint (outside the exception table's reach); false
// otherwise, for the caller to take ff_expf_core and the table.  Checked
// against the table-backed result on every float of the domain
// (umans_debug_expf_check, tests/test_gpu_refmath.py).
__device__ __forceinline__ bool exp_fast(float x, float band, float* out)
{
	const float kf = rintf(x * 92.33248138427734f);   // 64 / ln 2
	const float r_hi = fmaf(-kf, EXP_L1, x);
	const float r_lo = -kf * EXP_L2;
	const float rh = r_hi + r_lo;                       // TwoSum
	const float bb = rh - r_hi;
	const float rl = (r_hi - (rh - bb)) + (r_lo - bb);
	float c = fmaf(rh, 1.0f / 24.0f, 1.0f / 6.0f);
	c = fmaf(rh, c, 0.5f);
	const float q = fmaf(rh * rh, c, fmaf(rl, rh, rl));   // e^r - 1 - rh
	const int k = (int)kf;
	const int j = k & 63;
	const int kq = (k - j) / 64;                        // floor(k / 64)
	const float Th = FF_EXP2_TAB_D[j][0], Tl = FF_EXP2_TAB_D[j][1];
	const float Ph = Th * rh, Pl = fmaf(Th, rh, -Ph);   // Th rh exactly
	const float Sh = Th + Ph, Sl = Ph - (Sh - Th);      // Th + Ph exactly (|Ph| < Th)
	const float tail = Sl + (Pl + fmaf(Th, q, fmaf(Tl, rh, Tl)));
	const float f = Sh + tail;
	const float e = (Sh - f) + tail;                    // f's rounding residual
	const uint32_t fb = __float_as_uint(f);
	const float ulp = __uint_as_float((fb & 0x7f800000u) - (23u << 23));
	if ((fb & 0x007fffffu) == 0) return false;          // a power of two: unequal ulps on its two sides
	if (!(fabsf(e) < ulp * (0.5f - band - 0x1p-12f))) return false;
	*out = f * __uint_as_float((uint32_t)(kq + 127) << 23);   // kq in [-126, 0]: exact
	return true;
}

// The host C library's expf(x), exactly (see the header comment).
__device__ __forceinline__ float ref_expf(const ExpExceptions& T, float x)
{
	if (!(x >= FF_EXP_LO && x <= 0.0f)) return (float)exp((double)x);
	float yf;
	if (T.fast && exp_fast(x, T.band, &yf)) return yf;
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

// ---------------------------------------------------------------------------
// Reference-exact float sine and cosine.
//
// The reference takes sin/cos of float arguments, which resolve to the host C
// library's sinf/cosf: the gradient rotation (costFunction.cpp:30-34,
// FOEAvoidance.cpp:142), the random-sample rotation (costFunction.cpp:104 via
// rotateCounterClockwise, vector2D.h:166-170) and the segment collision time
// (costFunction.cpp:321).  The host sinf/cosf round ~1-3% of the arguments
// above 2^-5 the other way from the correctly rounded value (always within
// 0.061 ulp of a rounding midpoint), which the crowd dynamics amplify.  Same
// scheme as the exponential:
//  * ff_sincos_core: Cody-Waite reduction x = k pi/2 + r with pi/2 in four
//    floats (k * P1 exact for |k| < 2^12, |x| <= SC_LIMIT), then
//    r = j/64 + d, |d| <= 1/128, and
//      sin r = sin(j/64) cos d + cos(j/64) sin d,
//      cos r = cos(j/64) cos d - sin(j/64) sin d
//    with sin, cos(j/64) as float pairs (gen_sincos_table.py, 2^-48) and
//    cos d = 1 - d^2/2 + d^4/24, sin d = d - d^3/6 + d^5/120, all in
//    float-float (~2^-40 relative before the final rounding; only IEEE float
//    +,-,* and exact products, so host and device agree bit for bit);
//  * the host enumerates every float of |x| <= SC_LIMIT, records the
//    arguments where the C library differs, and the smallest distance of
//    such an argument's value from the rounding point (the "near" bound);
//  * the device looks the argument up only when its value lies that close
//    to a rounding midpoint (~1/8 of the calls), and returns the host
//    library's bits.
// Beyond SC_LIMIT the value is (float)sin((double)x), (float)cos((double)x).
constexpr float SC_LIMIT = 64.0f;
constexpr float SC_TINY = 0x1p-12f;     // below: sin x = x, cos x = 1 (correctly rounded)
constexpr float SC_P1 = 0x1.9220000000000p+0f;
constexpr float SC_P2 = -0x1.2aeef40000000p-18f;
constexpr float SC_P3 = -0x1.73dcb40000000p-43f;
constexpr float SC_P4 = 0x1.3198a20000000p-69f;
constexpr float SC_TWO_OVER_PI = 0x1.45f3060000000p-1f;

// { sin hi, sin lo, cos hi, cos lo } of j/64, j = 0..52
#if defined(__CUDACC__)
static __device__ const float SC_TAB_D[53][4] = {
	{ 0.0f, 0.0f, 0x1.0000000000000p+0f, 0.0f },
	{ 0x1.fffaaa0000000p-7f, 0x1.5dddda0000000p-32f, 0x1.fff0000000000p-1f, 0x1.5554a00000000p-29f },
	{ 0x1.ffeaaa0000000p-6f, 0x1.dddd0e0000000p-31f, 0x1.ffc0020000000p-1f, -0x1.555b060000000p-26f },
	{ 0x1.7fdc020000000p-5f, -0x1.f9a08a0000000p-30f, 0x1.ff70060000000p-1f, 0x1.7fbf340000000p-26f },
	{ 0x1.ffaaae0000000p-5f, 0x1.dda9dc0000000p-30f, 0x1.ff00160000000p-1f, -0x1.56c1660000000p-26f },
	{ 0x1.3facb20000000p-4f, -0x1.a5d1540000000p-29f, 0x1.fe70340000000p-1f, 0x1.29ef6e0000000p-29f },
	{ 0x1.7f70100000000p-4f, 0x1.92a8720000000p-31f, 0x1.fdc06c0000000p-1f, -0x1.0328ca0000000p-30f },
	{ 0x1.bf1b780000000p-4f, 0x1.5a0e480000000p-30f, 0x1.fcf0c80000000p-1f, 0x1.d336240000000p-34f },
	{ 0x1.feaaee0000000p-4f, 0x1.d0ddc60000000p-29f, 0x1.fc01560000000p-1f, -0x1.b054860000000p-26f },
	{ 0x1.1f0d3e0000000p-3f, -0x1.0a062a0000000p-28f, 0x1.faf2220000000p-1f, 0x1.8f12f40000000p-27f },
	{ 0x1.3eb3120000000p-3f, 0x1.8bacda0000000p-28f, 0x1.f9c3400000000p-1f, 0x1.4f98860000000p-26f },
	{ 0x1.5e44fc0000000p-3f, 0x1.f424de0000000p-28f, 0x1.f874c20000000p-1f, 0x1.c3dd9e0000000p-26f },
	{ 0x1.7dc1020000000p-3f, 0x1.f75e560000000p-28f, 0x1.f706be0000000p-1f, -0x1.84c7920000000p-31f },
	{ 0x1.9d252e0000000p-3f, -0x1.e6279e0000000p-28f, 0x1.f579480000000p-1f, 0x1.9fecf20000000p-26f },
	{ 0x1.bc6f840000000p-3f, 0x1.db8c340000000p-28f, 0x1.f3cc7c0000000p-1f, 0x1.d9e8b60000000p-28f },
	{ 0x1.db9e160000000p-3f, -0x1.2968c20000000p-33f, 0x1.f200740000000p-1f, -0x1.ef336c0000000p-26f },
	{ 0x1.faaeee0000000p-3f, -0x1.619d520000000p-28f, 0x1.f0154a0000000p-1f, -0x1.0422be0000000p-30f },
	{ 0x1.0cd00c0000000p-2f, 0x1.de6c860000000p-27f, 0x1.ee0b200000000p-1f, -0x1.0fc3ba0000000p-27f },
	{ 0x1.1c37d60000000p-2f, 0x1.31ae1e0000000p-28f, 0x1.ebe2140000000p-1f, 0x1.eeddf40000000p-26f },
	{ 0x1.2b8ddc0000000p-2f, 0x1.0fad280000000p-28f, 0x1.e99a4c0000000p-1f, 0x1.d3e6c20000000p-28f },
	{ 0x1.3ad12a0000000p-2f, -0x1.12c5840000000p-27f, 0x1.e733ea0000000p-1f, 0x1.93d3fa0000000p-33f },
	{ 0x1.4a00ca0000000p-2f, -0x1.3c30b80000000p-28f, 0x1.e4af140000000p-1f, 0x1.6548940000000p-26f },
	{ 0x1.591bca0000000p-2f, -0x1.7429a40000000p-32f, 0x1.e20bf40000000p-1f, 0x1.359ad80000000p-26f },
	{ 0x1.6821380000000p-2f, 0x1.471afe0000000p-27f, 0x1.df4ab40000000p-1f, -0x1.4278a20000000p-29f },
	{ 0x1.7710260000000p-2f, -0x1.5137be0000000p-27f, 0x1.dc6b7e0000000p-1f, 0x1.732b220000000p-26f },
	{ 0x1.85e7a20000000p-2f, -0x1.afb2d60000000p-27f, 0x1.d96e820000000p-1f, 0x1.ee353c0000000p-26f },
	{ 0x1.94a6be0000000p-2f, 0x1.3ea8d80000000p-27f, 0x1.d653f00000000p-1f, 0x1.cf90100000000p-27f },
	{ 0x1.a34c920000000p-2f, -0x1.9d799c0000000p-29f, 0x1.d31bf80000000p-1f, 0x1.b1af800000000p-26f },
	{ 0x1.b1d8300000000p-2f, 0x1.4c85860000000p-28f, 0x1.cfc6d00000000p-1f, -0x1.6b54980000000p-27f },
	{ 0x1.c048b20000000p-2f, -0x1.09d7ec0000000p-27f, 0x1.cc54aa0000000p-1f, 0x1.594b980000000p-28f },
	{ 0x1.ce9d2e0000000p-2f, 0x1.ea52900000000p-29f, 0x1.c8c5c00000000p-1f, -0x1.cc795e0000000p-27f },
	{ 0x1.dcd4c20000000p-2f, -0x1.59ac6c0000000p-27f, 0x1.c51a480000000p-1f, 0x1.7162ec0000000p-26f },
	{ 0x1.eaee880000000p-2f, -0x1.769f420000000p-27f, 0x1.c152800000000p-1f, 0x1.96df540000000p-27f },
	{ 0x1.f8e99e0000000p-2f, 0x1.daaf260000000p-28f, 0x1.bd6ea40000000p-1f, -0x1.dfad620000000p-26f },
	{ 0x1.0362940000000p-1f, -0x1.8e59aa0000000p-27f, 0x1.b96eee0000000p-1f, 0x1.eb10820000000p-26f },
	{ 0x1.0a40220000000p-1f, -0x1.61f0000000000p-29f, 0x1.b553a40000000p-1f, 0x1.0c104e0000000p-29f },
	{ 0x1.110d0c0000000p-1f, 0x1.2da70e0000000p-27f, 0x1.b11d040000000p-1f, 0x1.62a4c60000000p-29f },
	{ 0x1.17c8e60000000p-1f, -0x1.a224a00000000p-30f, 0x1.accb520000000p-1f, 0x1.bda77a0000000p-27f },
	{ 0x1.1e73440000000p-1f, -0x1.b935160000000p-26f, 0x1.a85ed40000000p-1f, 0x1.b9f0160000000p-28f },
	{ 0x1.250bba0000000p-1f, -0x1.90ee880000000p-26f, 0x1.a3d7d00000000p-1f, 0x1.a95ee80000000p-28f },
	{ 0x1.2b91de0000000p-1f, 0x1.5108440000000p-26f, 0x1.9f368e0000000p-1f, 0x1.b225f00000000p-26f },
	{ 0x1.32054c0000000p-1f, -0x1.d6e8760000000p-26f, 0x1.9a7b5a0000000p-1f, 0x1.b5328a0000000p-28f },
	{ 0x1.3865980000000p-1f, -0x1.753afa0000000p-26f, 0x1.95a67e0000000p-1f, 0x1.963f980000000p-34f },
	{ 0x1.3eb25e0000000p-1f, -0x1.9265580000000p-26f, 0x1.90b8480000000p-1f, -0x1.ec89420000000p-27f },
	{ 0x1.44eb380000000p-1f, 0x1.cf386a0000000p-29f, 0x1.8bb1060000000p-1f, -0x1.688dc00000000p-27f },
	{ 0x1.4b0fc40000000p-1f, 0x1.aaadd80000000p-27f, 0x1.8691080000000p-1f, 0x1.aef4d80000000p-26f },
	{ 0x1.511fa00000000p-1f, -0x1.4265720000000p-28f, 0x1.8158a40000000p-1f, -0x1.cdd2540000000p-26f },
	{ 0x1.571a6a0000000p-1f, -0x1.3254ca0000000p-26f, 0x1.7c08280000000p-1f, -0x1.ec35620000000p-30f },
	{ 0x1.5cffc20000000p-1f, -0x1.280e1e0000000p-26f, 0x1.769fec0000000p-1f, 0x1.9548480000000p-27f },
	{ 0x1.62cf4a0000000p-1f, -0x1.b794e20000000p-27f, 0x1.7120460000000p-1f, 0x1.f4eed00000000p-26f },
	{ 0x1.6888a40000000p-1f, 0x1.c269660000000p-26f, 0x1.6b89900000000p-1f, -0x1.5841280000000p-27f },
	{ 0x1.6e2b780000000p-1f, -0x1.dfa1100000000p-28f, 0x1.65dc200000000p-1f, -0x1.0a39a40000000p-28f },
	{ 0x1.73b7680000000p-1f, 0x1.bd4af00000000p-30f, 0x1.6018520000000p-1f, 0x1.bd58f80000000p-27f },
};
#endif
static const float SC_TAB_H[53][4] = {
	{ 0.0f, 0.0f, 0x1.0000000000000p+0f, 0.0f },
	{ 0x1.fffaaa0000000p-7f, 0x1.5dddda0000000p-32f, 0x1.fff0000000000p-1f, 0x1.5554a00000000p-29f },
	{ 0x1.ffeaaa0000000p-6f, 0x1.dddd0e0000000p-31f, 0x1.ffc0020000000p-1f, -0x1.555b060000000p-26f },
	{ 0x1.7fdc020000000p-5f, -0x1.f9a08a0000000p-30f, 0x1.ff70060000000p-1f, 0x1.7fbf340000000p-26f },
	{ 0x1.ffaaae0000000p-5f, 0x1.dda9dc0000000p-30f, 0x1.ff00160000000p-1f, -0x1.56c1660000000p-26f },
	{ 0x1.3facb20000000p-4f, -0x1.a5d1540000000p-29f, 0x1.fe70340000000p-1f, 0x1.29ef6e0000000p-29f },
	{ 0x1.7f70100000000p-4f, 0x1.92a8720000000p-31f, 0x1.fdc06c0000000p-1f, -0x1.0328ca0000000p-30f },
	{ 0x1.bf1b780000000p-4f, 0x1.5a0e480000000p-30f, 0x1.fcf0c80000000p-1f, 0x1.d336240000000p-34f },
	{ 0x1.feaaee0000000p-4f, 0x1.d0ddc60000000p-29f, 0x1.fc01560000000p-1f, -0x1.b054860000000p-26f },
	{ 0x1.1f0d3e0000000p-3f, -0x1.0a062a0000000p-28f, 0x1.faf2220000000p-1f, 0x1.8f12f40000000p-27f },
	{ 0x1.3eb3120000000p-3f, 0x1.8bacda0000000p-28f, 0x1.f9c3400000000p-1f, 0x1.4f98860000000p-26f },
	{ 0x1.5e44fc0000000p-3f, 0x1.f424de0000000p-28f, 0x1.f874c20000000p-1f, 0x1.c3dd9e0000000p-26f },
	{ 0x1.7dc1020000000p-3f, 0x1.f75e560000000p-28f, 0x1.f706be0000000p-1f, -0x1.84c7920000000p-31f },
	{ 0x1.9d252e0000000p-3f, -0x1.e6279e0000000p-28f, 0x1.f579480000000p-1f, 0x1.9fecf20000000p-26f },
	{ 0x1.bc6f840000000p-3f, 0x1.db8c340000000p-28f, 0x1.f3cc7c0000000p-1f, 0x1.d9e8b60000000p-28f },
	{ 0x1.db9e160000000p-3f, -0x1.2968c20000000p-33f, 0x1.f200740000000p-1f, -0x1.ef336c0000000p-26f },
	{ 0x1.faaeee0000000p-3f, -0x1.619d520000000p-28f, 0x1.f0154a0000000p-1f, -0x1.0422be0000000p-30f },
	{ 0x1.0cd00c0000000p-2f, 0x1.de6c860000000p-27f, 0x1.ee0b200000000p-1f, -0x1.0fc3ba0000000p-27f },
	{ 0x1.1c37d60000000p-2f, 0x1.31ae1e0000000p-28f, 0x1.ebe2140000000p-1f, 0x1.eeddf40000000p-26f },
	{ 0x1.2b8ddc0000000p-2f, 0x1.0fad280000000p-28f, 0x1.e99a4c0000000p-1f, 0x1.d3e6c20000000p-28f },
	{ 0x1.3ad12a0000000p-2f, -0x1.12c5840000000p-27f, 0x1.e733ea0000000p-1f, 0x1.93d3fa0000000p-33f },
	{ 0x1.4a00ca0000000p-2f, -0x1.3c30b80000000p-28f, 0x1.e4af140000000p-1f, 0x1.6548940000000p-26f },
	{ 0x1.591bca0000000p-2f, -0x1.7429a40000000p-32f, 0x1.e20bf40000000p-1f, 0x1.359ad80000000p-26f },
	{ 0x1.6821380000000p-2f, 0x1.471afe0000000p-27f, 0x1.df4ab40000000p-1f, -0x1.4278a20000000p-29f },
	{ 0x1.7710260000000p-2f, -0x1.5137be0000000p-27f, 0x1.dc6b7e0000000p-1f, 0x1.732b220000000p-26f },
	{ 0x1.85e7a20000000p-2f, -0x1.afb2d60000000p-27f, 0x1.d96e820000000p-1f, 0x1.ee353c0000000p-26f },
	{ 0x1.94a6be0000000p-2f, 0x1.3ea8d80000000p-27f, 0x1.d653f00000000p-1f, 0x1.cf90100000000p-27f },
	{ 0x1.a34c920000000p-2f, -0x1.9d799c0000000p-29f, 0x1.d31bf80000000p-1f, 0x1.b1af800000000p-26f },
	{ 0x1.b1d8300000000p-2f, 0x1.4c85860000000p-28f, 0x1.cfc6d00000000p-1f, -0x1.6b54980000000p-27f },
	{ 0x1.c048b20000000p-2f, -0x1.09d7ec0000000p-27f, 0x1.cc54aa0000000p-1f, 0x1.594b980000000p-28f },
	{ 0x1.ce9d2e0000000p-2f, 0x1.ea52900000000p-29f, 0x1.c8c5c00000000p-1f, -0x1.cc795e0000000p-27f },
	{ 0x1.dcd4c20000000p-2f, -0x1.59ac6c0000000p-27f, 0x1.c51a480000000p-1f, 0x1.7162ec0000000p-26f },
	{ 0x1.eaee880000000p-2f, -0x1.769f420000000p-27f, 0x1.c152800000000p-1f, 0x1.96df540000000p-27f },
	{ 0x1.f8e99e0000000p-2f, 0x1.daaf260000000p-28f, 0x1.bd6ea40000000p-1f, -0x1.dfad620000000p-26f },
	{ 0x1.0362940000000p-1f, -0x1.8e59aa0000000p-27f, 0x1.b96eee0000000p-1f, 0x1.eb10820000000p-26f },
	{ 0x1.0a40220000000p-1f, -0x1.61f0000000000p-29f, 0x1.b553a40000000p-1f, 0x1.0c104e0000000p-29f },
	{ 0x1.110d0c0000000p-1f, 0x1.2da70e0000000p-27f, 0x1.b11d040000000p-1f, 0x1.62a4c60000000p-29f },
	{ 0x1.17c8e60000000p-1f, -0x1.a224a00000000p-30f, 0x1.accb520000000p-1f, 0x1.bda77a0000000p-27f },
	{ 0x1.1e73440000000p-1f, -0x1.b935160000000p-26f, 0x1.a85ed40000000p-1f, 0x1.b9f0160000000p-28f },
	{ 0x1.250bba0000000p-1f, -0x1.90ee880000000p-26f, 0x1.a3d7d00000000p-1f, 0x1.a95ee80000000p-28f },
	{ 0x1.2b91de0000000p-1f, 0x1.5108440000000p-26f, 0x1.9f368e0000000p-1f, 0x1.b225f00000000p-26f },
	{ 0x1.32054c0000000p-1f, -0x1.d6e8760000000p-26f, 0x1.9a7b5a0000000p-1f, 0x1.b5328a0000000p-28f },
	{ 0x1.3865980000000p-1f, -0x1.753afa0000000p-26f, 0x1.95a67e0000000p-1f, 0x1.963f980000000p-34f },
	{ 0x1.3eb25e0000000p-1f, -0x1.9265580000000p-26f, 0x1.90b8480000000p-1f, -0x1.ec89420000000p-27f },
	{ 0x1.44eb380000000p-1f, 0x1.cf386a0000000p-29f, 0x1.8bb1060000000p-1f, -0x1.688dc00000000p-27f },
	{ 0x1.4b0fc40000000p-1f, 0x1.aaadd80000000p-27f, 0x1.8691080000000p-1f, 0x1.aef4d80000000p-26f },
	{ 0x1.511fa00000000p-1f, -0x1.4265720000000p-28f, 0x1.8158a40000000p-1f, -0x1.cdd2540000000p-26f },
	{ 0x1.571a6a0000000p-1f, -0x1.3254ca0000000p-26f, 0x1.7c08280000000p-1f, -0x1.ec35620000000p-30f },
	{ 0x1.5cffc20000000p-1f, -0x1.280e1e0000000p-26f, 0x1.769fec0000000p-1f, 0x1.9548480000000p-27f },
	{ 0x1.62cf4a0000000p-1f, -0x1.b794e20000000p-27f, 0x1.7120460000000p-1f, 0x1.f4eed00000000p-26f },
	{ 0x1.6888a40000000p-1f, 0x1.c269660000000p-26f, 0x1.6b89900000000p-1f, -0x1.5841280000000p-27f },
	{ 0x1.6e2b780000000p-1f, -0x1.dfa1100000000p-28f, 0x1.65dc200000000p-1f, -0x1.0a39a40000000p-28f },
	{ 0x1.73b7680000000p-1f, 0x1.bd4af00000000p-30f, 0x1.6018520000000p-1f, 0x1.bd58f80000000p-27f },
};

RM_HD float sc_tab(int j, int w)
{
#if defined(__CUDA_ARCH__)
	return SC_TAB_D[j][w];
#else
	return SC_TAB_H[j][w];
#endif
}

// sin x and cos x rounded to float (*s, *c) and the residuals of those
// roundings (*rs, *rc: float-float value minus the rounded value).
RM_HD void ff_sincos_core(float x, float* s, float* c, float* rs, float* rc)
{
	if (fabsf(x) < SC_TINY) {
		*s = x; *rs = -(x * x * x) * (1.0f / 6.0f);
		*c = 1.0f; *rc = -(x * x) * 0.5f;
		return;
	}
	// x = k pi/2 + r, r = rh + rl
	const float kf = rintf(x * SC_TWO_OVER_PI);
	const int k = (int)kf;
	const float t1 = x - kf * SC_P1;                 // both exact
	const FF q2 = ff_two_prod(kf, SC_P2);
	const FF q3 = ff_two_prod(kf, SC_P3);
	const FF a1 = ff_two_sum(t1, -q2.h);
	const FF a2 = ff_two_sum(a1.h, -q2.l);
	const FF a3 = ff_two_sum(a2.h, -q3.h);
	const float lo0 = ((a1.l + a2.l) + a3.l) - q3.l - kf * SC_P4;
	const FF r = ff_two_sum(a3.h, lo0);
	// r = j/64 + d
	const float jf = rintf(r.h * 64.0f);
	const int j = (int)jf;
	const FF d = ff_two_sum(r.h - jf * (1.0f / 64.0f), r.l);   // the difference is exact
	const int ja = j < 0 ? -j : j;
	const float sg = j < 0 ? -1.0f : 1.0f;
	const float Sh = sg * sc_tab(ja, 0), Sl = sg * sc_tab(ja, 1);
	const float Ch = sc_tab(ja, 2), Cl = sc_tab(ja, 3);
	// 1 - cos d = eh + el, sin d = d.h + sl
	const FF dd = ff_two_prod(d.h, d.h);
	const float eh = 0.5f * dd.h;
	const float el = (0.5f * dd.l + d.h * d.l) - dd.h * dd.h * (1.0f / 24.0f);
	const float s3 = (d.h * dd.h) * (1.0f / 6.0f) + dd.h * d.l * 0.5f - (d.h * dd.h) * dd.h * (1.0f / 120.0f);
	const float sl = d.l - s3;
	// sin r = S + C sin d - S (1 - cos d)
	float sr, srr;
	{
		const FF A = ff_two_prod(Ch, d.h);
		const FF B = ff_two_prod(Sh, eh);
		const FF t = ff_two_sum(Sh, A.h);
		const FF u = ff_two_sum(t.h, -B.h);
		const float rest = ((Sl + A.l) - B.l) + ((Ch * sl + Cl * d.h) - (Sh * el + Sl * eh));
		const float lo = (t.l + u.l) + rest;
		sr = u.h + lo;
		srr = lo - (sr - u.h);
	}
	// cos r = C - S sin d - C (1 - cos d)
	float cr, crr;
	{
		const FF A = ff_two_prod(Sh, d.h);
		const FF B = ff_two_prod(Ch, eh);
		const FF t = ff_two_sum(Ch, -A.h);
		const FF u = ff_two_sum(t.h, -B.h);
		const float rest = ((Cl - A.l) - B.l) - ((Sh * sl + Sl * d.h) + (Ch * el + Cl * eh));
		const float lo = (t.l + u.l) + rest;
		cr = u.h + lo;
		crr = lo - (cr - u.h);
	}
	switch (k & 3) {
	case 0: *s = sr; *rs = srr; *c = cr; *rc = crr; break;
	case 1: *s = cr; *rs = crr; *c = -sr; *rc = -srr; break;
	case 2: *s = -sr; *rs = -srr; *c = -cr; *rc = -crr; break;
	default: *s = -cr; *rs = -crr; *c = sr; *rc = srr; break;
	}
}

// |r| / (half the spacing of floats from f toward r), as a float: exact,
// since the spacing is a power of two.
RM_HD float sc_midpoint_ratio(float f, float r)
{
	const uint32_t b = rm_bits(f) & 0x7fffffffu;
	if (b < (25u << 23)) return 0.0f;    // |f| < 2^-102 (never reached above SC_TINY)
	float half = rm_float((b & 0x7f800000u) - (24u << 23));
	if ((b & 0x007fffffu) == 0 && ((r < 0.0f) != (f < 0.0f))) half *= 0.5f;
	return fabsf(r) / half;
}

// open-addressing tables of (argument bits, host sinf / cosf bits), key 0 =
// empty; sym: the host library is odd/even (sinf(-x) = -sinf(x),
// cosf(-x) = cosf(x) on the whole domain), the keys are |x|
struct SinCosExceptions {
	const uint2* sin_slots;
	const uint2* cos_slots;
	uint32_t sin_mask, cos_mask;
	int sin_shift, cos_shift;
	float sin_near, cos_near;   // look up when sc_midpoint_ratio >= this
	int sym;
};

#if defined(__CUDACC__)
__device__ __forceinline__ float sc_patch(const uint2* slots, uint32_t mask, int shift, int sym, bool odd, float x,
                                          float y)
{
	if (slots == nullptr) return y;   // tables not set on this device: the float-float value
	const uint32_t b = sym ? (__float_as_uint(x) & 0x7fffffffu) : __float_as_uint(x);
	uint32_t h = ff_hash(b, shift);
	for (;;) {
		const uint2 e = __ldg(&slots[h]);
		if (e.x == 0) return y;
		if (e.x == b) {
			const float v = __uint_as_float(e.y);
			return (sym && odd && x < 0.0f) ? -v : v;
		}
		h = (h + 1) & mask;
	}
}

// The host C library's sinf(x) and cosf(x), exactly for |x| <= SC_LIMIT.
__device__ __forceinline__ void ref_sincosf(const SinCosExceptions& T, float x, float* s, float* c)
{
	if (!(fabsf(x) <= SC_LIMIT)) {
		*s = (float)sin((double)x);
		*c = (float)cos((double)x);
		return;
	}
	float fs, fc, rs, rc;
	ff_sincos_core(x, &fs, &fc, &rs, &rc);
	if (sc_midpoint_ratio(fs, rs) >= T.sin_near) fs = sc_patch(T.sin_slots, T.sin_mask, T.sin_shift, T.sym, true, x, fs);
	if (sc_midpoint_ratio(fc, rc) >= T.cos_near) fc = sc_patch(T.cos_slots, T.cos_mask, T.cos_shift, T.sym, false, x, fc);
	*s = fs;
	*c = fc;
}
__device__ __forceinline__ float ref_sinf(const SinCosExceptions& T, float x)
{
	if (!(fabsf(x) <= SC_LIMIT)) return (float)sin((double)x);
	float fs, fc, rs, rc;
	ff_sincos_core(x, &fs, &fc, &rs, &rc);
	if (sc_midpoint_ratio(fs, rs) >= T.sin_near) fs = sc_patch(T.sin_slots, T.sin_mask, T.sin_shift, T.sym, true, x, fs);
	return fs;
}
#endif

// host side (refmath.cpp): table shared by all simulations on a device
bool sincos_exceptions_for_device(SinCosExceptions* out, size_t* count, std::string& err);

// ---------------------------------------------------------------------------
// getLineIntersection (vector2D.h:249-272) without FP64 in the common case.
//
// The reference intersects lines in double: a1, b1, a2, b2 are float
// differences, c1, c2 and the determinant sums of exact products rounded to
// double, the result coordinates (b2 c1 - b1 c2) / det and (a1 c2 - a2 c1) /
// det rounded to double and then to float.  FP64 is slow on this GPU, and
// Paris evaluates the intersection for every (sample, neighbour) pair.  The
// same expressions are evaluated here in float-float arithmetic (~2^-46),
// with a bound on the distance between that value and the double
// pipeline's (both within a few 2^-46 of the exact value, amplified by the
// cancellation in det and in the numerators).  When the float rounding of
// every value within the bound is the same, and the parallel-lines test is
// decided outside its own bound, the float-float result is the reference's;
// otherwise the caller evaluates the double pipeline (line_intersection_d).

// the double pipeline, as the reference evaluates it (no contraction)
RM_HD bool line_intersection_d(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy,
                               float* rx, float* ry)
{
	const double a1 = (double)(by - ay), b1 = (double)(ax - bx);
	const double c1 = a1 * (double)ax + b1 * (double)ay;
	const double a2 = (double)(dy - cy), b2 = (double)(cx - dx);
	const double c2 = a2 * (double)cx + b2 * (double)cy;
	const double det = a1 * b2 - a2 * b1;
	if (fabs(det) < 0.00001) return false;
	*rx = (float)((b2 * c1 - b1 * c2) / det);
	*ry = (float)((a1 * c2 - a2 * c1) / det);
	return true;
}

RM_HD FF ff_add2(FF x, FF y)
{
	const FF s = ff_two_sum(x.h, y.h);
	return ff_two_sum(s.h, s.l + (x.l + y.l));
}
RM_HD FF ff_mulf(FF x, float b)
{
	const FF p = ff_two_prod(x.h, b);
	return ff_fast_two_sum(p.h, p.l + x.l * b);
}
RM_HD FF ff_div2(FF n, FF d)
{
	const float q1 = n.h / d.h;
	const FF p = ff_two_prod(q1, d.h);
	const FF r = ff_add2(n, FF{ -p.h, -(p.l + q1 * d.l) });
	return ff_fast_two_sum(q1, r.h / d.h);
}
// true when every value within `bound` of v rounds to the float v.h
RM_HD bool ff_rounds_to_h(FF v, float bound)
{
	const uint32_t b = rm_bits(v.h) & 0x7fffffffu;
	if (b < (40u << 23) || b >= 0x7e800000u) return false;   // |v| < 2^-87 or > 2^126, inf, nan
	float half = rm_float((b & 0x7f800000u) - (24u << 23));
	if ((b & 0x007fffffu) == 0) half *= 0.5f;                 // finer spacing below a power of two
	return half - fabsf(v.l) > bound;
}

// 1: intersection (*rx, *ry), 0: parallel, -1: undecided (use the double pipeline)
RM_HD int line_intersection_ff(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy,
                               float* rx, float* ry)
{
	const float a1 = by - ay, b1 = ax - bx, a2 = dy - cy, b2 = cx - dx;
	const FF c1 = ff_add2(ff_two_prod(a1, ax), ff_two_prod(b1, ay));
	const FF c2 = ff_add2(ff_two_prod(a2, cx), ff_two_prod(b2, cy));
	const FF p = ff_two_prod(a1, b2), q = ff_two_prod(a2, b1);
	const FF det = ff_add2(p, FF{ -q.h, -q.l });
	// magnitudes for the error bounds (float estimates; the 2^-43 factor is
	// ~8x the float-float and double error constants)
	const float TINY = 0x1p-100f;
	const float Mc1 = fabsf(a1 * ax) + fabsf(b1 * ay) + TINY;
	const float Mc2 = fabsf(a2 * cx) + fabsf(b2 * cy) + TINY;
	const float Mdet = fabsf(p.h) + fabsf(q.h) + TINY;
	const float adet = fabsf(det.h);
	const float T = 1e-5f;
	const float margin = 0x1p-43f * Mdet + 0x1p-20f * T;
	if (adet < T - margin) return 0;
	if (!(adet > T + margin)) return -1;
	const FF nx = ff_add2(ff_mulf(c1, b2), ff_mulf(c2, -b1));
	const FF ny = ff_add2(ff_mulf(c2, a1), ff_mulf(c1, -a2));
	const FF X = ff_div2(nx, det), Y = ff_div2(ny, det);
	const float kdet = Mdet / adet + 1.0f;
	const float Bx = 0x1p-43f * ((fabsf(b2) * Mc1 + fabsf(b1) * Mc2) / adet + fabsf(X.h) * kdet);
	const float By = 0x1p-43f * ((fabsf(a1) * Mc2 + fabsf(a2) * Mc1) / adet + fabsf(Y.h) * kdet);
	if (!ff_rounds_to_h(X, Bx) || !ff_rounds_to_h(Y, By)) return -1;
	*rx = X.h;
	*ry = Y.h;
	return 1;
}

// ---------------------------------------------------------------------------
// (float)exp(-0.5 * ((double)a * a + (double)b * b)): the Gaussians of TtcaDca
// (TtcaDca.cpp:40-43 and :54-60), evaluated in double by the reference.  The
// squares are exact in float-float, their sum within 2^-47, so the argument
// is within 2^-46 |x| of the double one; the float-float exponential
// (ff_exp_ff) is then rounded to float when every value within the combined
// bound rounds the same way, else the double expression is evaluated.
RM_HD float exp_gauss(float a, float b)
{
	const FF q = ff_add2(ff_two_prod(a, a), ff_two_prod(b, b));
	const float xh = -0.5f * q.h, xl = -0.5f * q.l;
	if (xh < -104.5f) return 0.0f;    // below 2^-150.7: the float rounding is 0
	if (xh >= FF_EXP_LO && xh <= 0.0f) {
		float hi, lo, sc;
		ff_exp_ff(xh, xl, &hi, &lo, &sc);
		const float f = hi + lo;
		const FF v = FF{ f, lo - (f - hi) };
		const float bound = (0x1p-45f * fabsf(xh) + 0x1p-41f) * f;
		if (ff_rounds_to_h(v, bound)) return f * sc;
	}
	const double ad = (double)a, bd = (double)b;
	return (float)exp(-0.5 * (ad * ad + bd * bd));
}

}  // namespace umans
