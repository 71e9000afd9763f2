// Test harness (CPU): the GAF formatter's number formatting (graphaligner_gb300/csrc/gaf_format.cuh)
// against std::ostream's default double formatting and integer formatting, on the values GAF
// lines hold (X-scores / 100, match ratios and one minus them) and on doubles across the whole
// exponent range.  Prints "checked N mismatches M" and the first mismatches.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include "../../graphaligner_gb300/csrc/gaf_format.cuh"

static int bad = 0;
static long checked = 0;

static void check(double v)
{
    std::stringstream s;
    s << v;
    char buf[64];
    const int n = gaf::fmt_g(v, buf);
    const std::string mine(buf, n);
    checked++;
    if (mine != s.str() && bad++ < 20)
    {
        char hex[32];
        uint64_t b;
        memcpy(&b, &v, 8);
        snprintf(hex, sizeof hex, "%016llx", (unsigned long long)b);
        std::cout << "mismatch " << hex << " stream " << s.str() << " mine " << mine << "\n";
    }
}

int main()
{
    std::mt19937_64 rng(7);
    // X-scores / 100 of every alignment length and score a read of up to 1 Mbp gives, sampled
    for (int64_t x = -200000; x <= 200000; x++) check((double)(int32_t)x / 100.0);
    for (int k = 0; k < 1000000; k++) check((double)(int32_t)(rng() % 200000000) / 100.0 * ((rng() & 1) ? 1 : -1));
    // identity and divergence: matches / length and 1 - that
    for (uint64_t len = 1; len <= 3000; len++)
        for (uint64_t m = 0; m <= len; m += (len > 300 ? 7 : 1))
        {
            const double id = (double)m / (double)len;
            check(id);
            check(1.0 - id);
        }
    for (int k = 0; k < 1000000; k++)
    {
        const uint64_t len = 1 + rng() % 5000000, m = rng() % (len + 1);
        check((double)m / (double)len);
        check(1.0 - (double)m / (double)len);
    }
    // ties and carries at six digits, powers of ten, and random bit patterns over every exponent
    const double special[] = { 0.0, -0.0, 1.0, 0.5, 123456.5, 123457.5, 999999.5, 9999995.0, 0.0001, 0.00001, 1e-5, 99999.95, 1e6, 1e15,
        1e-300, 5e-324, 1.7976931348623157e308, 2.2250738585072014e-308, 0.1, 0.2, 0.3 };
    for (double v : special)
    {
        check(v);
        check(-v);
    }
    for (int p = -320; p <= 308; p++)
    {
        const double v = std::pow(10.0, p);
        check(v);
        check(std::nextafter(v, 0.0));
        check(std::nextafter(v, INFINITY));
    }
    for (int k = 0; k < 1500000; k++)
    {
        uint64_t b = rng();
        double v;
        memcpy(&v, &b, 8);
        if (std::isnan(v) || std::isinf(v)) continue;
        check(v);
    }
    // integers
    for (int k = 0; k < 1000000; k++)
    {
        const int64_t x = (int64_t)rng();
        char buf[32];
        const int n = gaf::fmt_i64(x, buf);
        if (std::string(buf, n) != std::to_string(x) && bad++ < 20) std::cout << "int mismatch " << x << "\n";
        checked++;
    }
    std::cout << "checked " << checked << " mismatches " << bad << "\n";
    return bad != 0;
}
