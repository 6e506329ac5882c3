// Host-side check of cal_div_small (c = 1..9), cal_div_recip (b = sqrt(2)),
// cal_le, cal_gt and cal_pos against the host's IEEE division and
// comparisons.  Usage: exact_div_check <n_random> <seed>
// Prints the number of mismatches (0 expected).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../opencal_gb300/csrc/models/exact_div.cuh"

static uint64_t s_state;
static uint64_t next_u64()
{
    uint64_t z = (s_state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static bool same(double a, double b)
{
    uint64_t x, y;
    memcpy(&x, &a, 8);
    memcpy(&y, &b, 8);
    return x == y || (a != a && b != b);
}

int main(int argc, char** argv)
{
    long n = argc > 1 ? atol(argv[1]) : 10000000;
    s_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    long bad = 0;
    const double rb_b = std::sqrt(2.0), rb_y = 1.0 / rb_b;
    if (!cal_recip_exact_ok(rb_b, rb_y)) {
        printf("reciprocal precondition fails for sqrt(2)\n");
        return 1;
    }
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 3.0, 5.0, 15.0, 1e-310, -1e-310, 2.2250738585072014e-308,
                               1e308, 1.7976931348623157e308, INFINITY, -INFINITY, NAN, 0.1, 1.0 / 3.0,
                               4503599627370496.0, 9007199254740991.0, 1e-300, 6.0e-305};
    for (double x : specials)
        for (int c = 1; c <= 9; c++)
            if (!same(cal_div_small(x, c), x / (double)c)) {
                if (bad < 10) printf("special x=%a c=%d got %a want %a\n", x, c, cal_div_small(x, c), x / (double)c);
                bad++;
            }
    for (long k = 0; k < n; k++) {
        uint64_t r = next_u64();
        double x;
        if (k & 1) {
            /* random bit patterns: every exponent and significand */
            memcpy(&x, &r, 8);
        } else {
            /* values of the model's range: sums of thicknesses and altitudes */
            x = (double)(r >> 11) * (1.0 / 9007199254740992.0) * 4000.0 - 200.0;
        }
        int c = 1 + (int)(next_u64() % 9);
        if (!same(cal_div_small(x, c), x / (double)c)) {
            if (bad < 10) printf("x=%a c=%d got %a want %a\n", x, c, cal_div_small(x, c), x / (double)c);
            bad++;
        }
        double y;
        uint64_t r2 = next_u64();
        if (k & 2)
            memcpy(&y, &r2, 8);
        else
            y = x + (double)((int64_t)(r2 % 7) - 3) * (std::fabs(x) * 1e-16);
        if (cal_le(x, y) != (x <= y) || cal_gt(x, y) != (x > y) || cal_pos(x) != (x > 0)) {
            if (bad < 10) printf("compare x=%a y=%a\n", x, y);
            bad++;
        }
        if (!same(cal_div_recip(x, rb_b, rb_y), x / rb_b)) {
            if (bad < 10) printf("recip x=%a got %a want %a\n", x, cal_div_recip(x, rb_b, rb_y), x / rb_b);
            bad++;
        }
    }
    printf("%ld\n", bad);
    return bad != 0;
}
