// Host check of cube_node's float-reciprocal decode (meshoid_gb300/csrc/
// mg_cube.cuh): for cubes of fewer than 2^22 nodes it must agree with integer
// division at every index; checked at every index of small cubes and at the
// column boundaries (m nz - 1, m nz, and the same for ny) plus random indices
// of large ones.  Built and run on the CPU by tests/test_native_helpers.py.
#include <stdint.h>
#include <stdio.h>

#include "mg_cube.cuh"

using namespace mg;

static uint64_t rng_state = 0x94D049BB133111EBull;
static uint64_t urand64() {
    rng_state ^= rng_state >> 12;
    rng_state ^= rng_state << 25;
    rng_state ^= rng_state >> 27;
    return rng_state * 2685821657736338717ull;
}

static int check(int nx, int ny, int nz, int64_t c) {
    const int64_t total = (int64_t)nx * ny * nz;
    const CubeDiv d = cube_div(ny, nz, total);
    int i, j, l;
    cube_node(c, d, i, j, l);
    const int64_t col = c / nz;
    const int ri = (int)(col / ny), rj = (int)(col % ny), rl = (int)(c % nz);
    if (i != ri || j != rj || l != rl) {
        printf("  cube %d x %d x %d index %lld: (%d %d %d) instead of (%d %d %d)\n", nx, ny, nz, (long long)c, i, j, l,
               ri, rj, rl);
        return 1;
    }
    return 0;
}

int main() {
    int fails = 0;
    long long checked = 0;
    // every index of every cube up to 24 nodes a side
    for (int nx = 1; nx <= 24 && fails < 10; ++nx)
        for (int ny = 1; ny <= 24; ++ny)
            for (int nz = 1; nz <= 24; ++nz)
                for (int64_t c = 0; c < (int64_t)nx * ny * nz; ++c, ++checked) fails += check(nx, ny, nz, c);
    // large cubes below 2^22 nodes: column boundaries and random indices
    for (int t = 0; t < 20000 && fails < 10; ++t) {
        const int nz = 1 + (int)(urand64() % 4096), ny = 1 + (int)(urand64() % 4096);
        int64_t maxx = ((1ll << 22) - 1) / ((int64_t)ny * nz);
        if (maxx < 1) continue;
        const int nx = 1 + (int)(urand64() % (uint64_t)maxx);
        const int64_t total = (int64_t)nx * ny * nz;
        for (int s = 0; s < 64; ++s) {
            const int64_t m = (int64_t)(urand64() % (uint64_t)(total / nz + 1));
            const int64_t cs[4] = {m * nz - 1, m * nz, m * nz + nz - 1, (int64_t)(urand64() % (uint64_t)total)};
            for (int64_t c : cs)
                if (c >= 0 && c < total) { fails += check(nx, ny, nz, c); ++checked; }
            const int64_t mc = (int64_t)(urand64() % (uint64_t)(nx + 1)) * ny * nz - 1;  // last node of a plane
            if (mc >= 0 && mc < total) { fails += check(nx, ny, nz, mc); ++checked; }
        }
    }
    printf("cube_node: %lld indices checked, %d wrong\n", checked, fails);
    printf(fails ? "FAILED\n" : "ok\n");
    return fails ? 1 : 0;
}
