// Compares the device STL number converter (compiled here as host code) with
// strtod: every number the converter accepts as exact must have strtod's
// bits.  Usage: stlnum_check N SEED -> "checked <n> exact <m>" or the first
// mismatch.
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

#include "stl_number.h"

static bool check(const std::string& s, long* exact) {
    double v = 0.0;
    bool ex = false;
    const char* e = lbm::stlnum::parse_number(s.data(), s.data() + s.size(), &v, &ex);
    char* end = nullptr;
    const double ref = std::strtod(s.c_str(), &end);
    if (!e) {
        std::printf("MISMATCH no number parsed: '%s'\n", s.c_str());
        return false;
    }
    if ((size_t)(e - s.data()) != (size_t)(end - s.c_str())) {
        std::printf("MISMATCH end '%s': %td vs %td\n", s.c_str(), e - s.data(), end - s.c_str());
        return false;
    }
    if (!ex) return true;
    ++*exact;
    uint64_t a, b;
    std::memcpy(&a, &v, 8);
    std::memcpy(&b, &ref, 8);
    if (a != b) {
        std::printf("MISMATCH '%s': %.17g (%016" PRIx64 ") vs strtod %.17g (%016" PRIx64 ")\n", s.c_str(), v, a, ref, b);
        return false;
    }
    return true;
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 100000;
    std::mt19937_64 rng(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
    long exact = 0, checked = 0;
    const char* fixed[] = {"0", "-0", "0.1", "1", "9007199254740993", "9007199254740992", "9007199254740994",
                           "9007199254740995", "18014398509481985", "1e-27", "1e27", "9999999999999999999",
                           "9999999999999999999e27", "1.0000000000000000000", "123456789012345678e-27",
                           "2.2250738585072014e-27", "4.9406564584124654", "0.30000000000000004",
                           "1.7976931348623157", "+.5", "5.", "1.e3", "-7.25E+02", "1e", "1e+", "3.14159265358979323846",
                           "0.000000000000000000000000001", "123.456e-5", "1.5e-0", "-1.2246467991473532e-16",
                           "6.123233995736766e-17", "1e-60", "9999999999999999999e-60", "1e60", "1e33",
                           "9999999999999999999e41", "4.4501477170144023e-28", "2.4703282292062327e-20"};
    for (const char* f : fixed) {
        ++checked;
        if (!check(f, &exact)) return 1;
    }
    char buf[128];
    for (long i = 0; i < n; ++i) {
        const int kind = (int)(rng() % 4);
        const int nd = 1 + (int)(rng() % 19);
        uint64_t w = 0;
        for (int d = 0; d < nd; ++d) w = w * 10 + rng() % 10;
        const int pt = (int)(rng() % (nd + 1));
        std::string digs = std::to_string(w);
        while ((int)digs.size() < nd) digs = "0" + digs;
        std::string s = (rng() & 1) ? "-" : "";
        s += digs.substr(0, pt).empty() ? "0" : digs.substr(0, pt);
        if (pt < nd) s += "." + digs.substr(pt);
        if (kind == 1) { std::snprintf(buf, sizeof buf, "e%+d", (int)(rng() % 121) - 60); s += buf; }
        if (kind == 2) {
            // printf forms STL writers use
            const double x = std::ldexp((double)(rng() >> 11), (int)(rng() % 200) - 180);
            const int prec = (int)(rng() % 18);
            const int form = (int)(rng() % 3);
            std::snprintf(buf, sizeof buf, form == 0 ? "%.*e" : (form == 1 ? "%.*f" : "%.*g"), form == 2 ? 17 : prec,
                          (rng() & 1) ? x : -x);
            s = buf;
        }
        if (kind == 3) {
            // halfway and near-halfway integers above 2^53
            const uint64_t m = (rng() >> 11) | (1ull << 52);
            const uint64_t v = (m << 1) + (rng() % 3);
            std::snprintf(buf, sizeof buf, "%" PRIu64 "e%d", v, (int)(rng() % 9) - 4);
            s = buf;
        }
        ++checked;
        if (!check(s, &exact)) return 1;
    }
    std::printf("checked %ld exact %ld\n", checked, exact);
    return 0;
}
