// Host check of the site-coordinate division of lattice.cuh: div_n with the
// multiplier and shift of div_magic equals s / n for divisors 1..4096, every
// power of two up to 2^30 and its neighbours, and sampled large divisors, at
// the site indices around every multiple of n that matters (0, n - 1, n,
// n + 1, the last multiples below 2^31) and at pseudo-random ones.
#include <cstdio>

#include "../openpixi_gb300/csrc/lattice.cuh"

static unsigned long long rng = 0x9E3779B97F4A7C15ULL;
static unsigned next_u31() {
    rng = rng * 6364136223846793005ULL + 1442695040888963407ULL;
    return (unsigned)(rng >> 33);  // 31 bits
}

static int check(int n, long *count) {
    opx::Lat L = {};
    opx::div_magic(n, &L.dmul[0], &L.dsh[0]);
    opx::div_magic(n, &L.dmul[1], &L.dsh[1]);
    const long top = 2147483647L;
    long cand[16] = {0, 1, n - 1L, n, n + 1L, 2L * n - 1, 2L * n, top, top - 1, (top / n) * n, (top / n) * n - 1,
                     (top / n) * n + (n - 1L), 12345L * n, 12345L * n - 1, 777L * n + n / 2, 3L * n + 1};
    for (long s : cand) {
        if (s < 0 || s > top) continue;
        for (int k = 0; k < 2; k++) {
            if (opx::div_n(L, k, (int)s) != (int)(s / n)) {
                std::printf("mismatch n=%d s=%ld\n", n, s);
                return 1;
            }
            (*count)++;
        }
    }
    for (int r = 0; r < 256; r++) {
        const int s = (int)next_u31();
        if (opx::div_n(L, 0, s) != s / n) {
            std::printf("mismatch n=%d s=%d\n", n, s);
            return 1;
        }
        (*count)++;
    }
    return 0;
}

int main() {
    long count = 0;
    for (int n = 1; n <= 4096; n++)
        if (check(n, &count)) return 1;
    for (int e = 1; e <= 30; e++)
        for (int d = -1; d <= 1; d++)
            if (check((1 << e) + d, &count)) return 1;
    for (int r = 0; r < 2000; r++)
        if (check(1 + (int)(next_u31() % 2147483646u), &count)) return 1;
    std::printf("ok %ld\n", count);
    return 0;
}
