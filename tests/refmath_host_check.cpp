// Host check of the reference-exact arithmetic in refmath.hpp (compiled and
// run by test_refmath_host.py):
//  * line_intersection_ff either declines or equals the reference's double
//    pipeline, on Paris-like, obstacle-like and adversarial inputs;
//  * ff_sincos_core differs from the C library's sinf/cosf only at arguments
//    whose value lies close to a rounding midpoint (the only ones the device
//    looks up);
//  * exp_gauss equals the double expression it stands for.
#include "../umans_gb300/csrc/refmath.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using namespace umans;

int main(int argc, char** argv)
{
	const long per_mode = argc > 1 ? std::atol(argv[1]) : 1000000;
	std::mt19937_64 g(7);
	std::uniform_real_distribution<float> U(-1, 1);
	long n = 0, declined = 0, bad = 0;
	for (int mode = 0; mode < 5; ++mode)
		for (long i = 0; i < per_mode; ++i) {
			float ax, ay, bx, by, cx, cy, dx, dy;
			const float an = 3.14159f * U(g), bn = 3.14159f * U(g);
			if (mode == 0) {   // Paris: position, position + unit direction, neighbour, neighbour + velocity
				ax = 200 * U(g); ay = 200 * U(g);
				float ux = std::cos(an), uy = std::sin(an);
				const float l = std::sqrt(ux * ux + uy * uy);
				bx = ax + ux / l; by = ay + uy / l;
				cx = ax + 5 * U(g); cy = ay + 5 * U(g); dx = cx + 2 * U(g); dy = cy + 2 * U(g);
			} else if (mode == 1) {   // obstacles: position, position + velocity, segment ends
				ax = 20 * U(g); ay = 20 * U(g); bx = ax + 2 * U(g); by = ay + 2 * U(g);
				cx = 20 * U(g); cy = 20 * U(g); dx = 20 * U(g); dy = 20 * U(g);
			} else if (mode == 2) {   // nearly parallel
				ax = 50 * U(g); ay = 50 * U(g); bx = ax + std::cos(an); by = ay + std::sin(an);
				cx = ax + 3 * U(g); cy = ay + 3 * U(g);
				const float e = 1e-4f * U(g), s = U(g);
				dx = cx + std::cos(an + e) * s; dy = cy + std::sin(an + e) * s;
			} else if (mode == 3) {   // intersection near the origin, points far along the lines
				const float x0 = 1e-3f * U(g), y0 = 1e-3f * U(g), t = 100 * U(g), s = 100 * U(g);
				ax = x0 + t * std::cos(an); ay = y0 + t * std::sin(an); bx = ax + std::cos(an); by = ay + std::sin(an);
				cx = x0 + s * std::cos(bn); cy = y0 + s * std::sin(bn); dx = cx + std::cos(bn); dy = cy + std::sin(bn);
			} else {   // determinant at the 1e-5 threshold
				ax = 10 * U(g); ay = 10 * U(g); bx = ax + 1; by = ay;
				cx = 10 * U(g); cy = 10 * U(g); dx = cx + U(g); dy = cy - 1e-5f * (1 + 1e-3f * U(g));
			}
			float rx = 0, ry = 0, fx = 0, fy = 0;
			const bool ok = line_intersection_d(ax, ay, bx, by, cx, cy, dx, dy, &rx, &ry);
			const int r = line_intersection_ff(ax, ay, bx, by, cx, cy, dx, dy, &fx, &fy);
			++n;
			if (r < 0) { ++declined; continue; }
			if ((r == 1) != ok || (ok && (fx != rx || fy != ry))) ++bad;
		}
	std::printf("isect n=%ld declined=%ld mismatches=%ld\n", n, declined, bad);

	// sine / cosine: every argument where the core and the library differ
	// must have a midpoint ratio of at least 0.75
	long m = 0, diff = 0, unflagged = 0;
	std::uniform_real_distribution<float> A(-64, 64);
	for (long i = 0; i < 4 * per_mode; ++i) {
		const float x = (i & 1) ? A(g) : std::ldexp(U(g), -(int)(i % 20));
		float s, c, rs, rc;
		ff_sincos_core(x, &s, &c, &rs, &rc);
		const float ls = sinf(x), lc = cosf(x);
		++m;
		if (s != ls) { ++diff; unflagged += sc_midpoint_ratio(s, rs) < 0.75f; }
		if (c != lc) { ++diff; unflagged += sc_midpoint_ratio(c, rc) < 0.75f; }
	}
	std::printf("sincos n=%ld differ=%ld unflagged=%ld\n", m, diff, unflagged);

	long ge = 0, gbad = 0;
	std::uniform_real_distribution<float> G(0, 1);
	for (long i = 0; i < 4 * per_mode; ++i) {
		const float sc = (i & 3) == 0 ? 0.1f : ((i & 3) == 1 ? 3.0f : ((i & 3) == 2 ? 15.0f : 40.0f));
		const float a = sc * G(g), b = (i & 4) ? 0.0f : sc * G(g);
		const double ad = a, bd = b;
		const float want = (float)std::exp(-0.5 * (ad * ad + bd * bd));
		++ge;
		if (exp_gauss(a, b) != want) ++gbad;
	}
	std::printf("gauss n=%ld mismatches=%ld\n", ge, gbad);
	return (bad == 0 && unflagged == 0 && gbad == 0) ? 0 : 1;
}
