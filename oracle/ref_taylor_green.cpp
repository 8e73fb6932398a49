// Test-infrastructure harness: evaluates the reference's analytic Taylor-Green
// solution (tests/validation/analytical/TaylorGreenSolution.h:25-47, compiled
// in place by oracle/Makefile.ref, which only decodes the three HTML entities
// the header is stored with: &lt; &gt; &amp;) on a seeded set of points and
// times, and writes them for tests/golden/make_taylor_green.py.
// Output records (little-endian doubles): x, y, z, t, Re, u, v, w, E(t, Re).
#include <cstdio>
#include <random>

#include "TaylorGreenSolution.h"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    std::mt19937_64 rng(20241204ULL);
    std::uniform_real_distribution<double> pos(0.0, 6.283185307179586), tim(0.0, 3.0), re(5.0, 500.0);
    const int n = 2048;
    std::fwrite(&n, 4, 1, f);
    for (int i = 0; i < n; ++i) {
        double r[9];
        r[0] = pos(rng); r[1] = pos(rng);
        r[2] = (i % 2) ? pos(rng) : 0.0;  // half on the z = 0 plane (the 2-D vortex)
        r[3] = tim(rng); r[4] = re(rng);
        fluidloom::validation::TaylorGreenSolution::computeVelocity(r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7]);
        r[8] = fluidloom::validation::TaylorGreenSolution::computeKineticEnergy(r[3], r[4]);
        std::fwrite(r, 8, 9, f);
    }
    std::fclose(f);
    return 0;
}
