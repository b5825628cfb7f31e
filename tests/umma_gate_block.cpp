// Host check of the gate block of a complex128 tensor-memory pass, built by
// libhqs.so (plan_launches + write_umma_pool): every gate real is decoded
// from the fp16 digit planes at the row and 16-byte chunk the MMAs read
// (128-byte swizzle: chunk c of row r at chunk c ^ (r mod 8)), in both row
// orders: plane-major (row 64 j + n, passes with diagonal runs) and by output
// half (row 192 h + 32 j + n mod 32, passes that hold only the dense gate).
// The digits rebuild each real of the gate's real form to one unit of its
// column's 54-bit grid; the column exponents are the columns' largest.
// Prints one line per case: "<case> halves=<0|1> max_units=<x> ok".
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "workspace.h"

namespace {

double f16_value(uint16_t h) {
    const int e = (h >> 10) & 0x1F, m = h & 0x3FF;
    const double v = e == 0 ? std::ldexp((double)m, -24) : std::ldexp((double)(m | 0x400), e - 25);
    return (h & 0x8000) ? -v : v;
}

int biased_exponent(double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return (int)((u >> 52) & 0x7FF);
}

// the gate's real form: y = x B for interleaved (re, im) inputs and outputs
double real_form(const hqs::GateOp& g, int kk, int nn) {
    const hqs::cplx m = g.m[(size_t)(nn >> 1) * 32 + (size_t)(kk >> 1)];
    if ((kk & 1) == 0) return (nn & 1) == 0 ? m.real() : m.imag();
    return (nn & 1) == 0 ? -m.imag() : m.real();
}

int check(const char* name, const std::vector<hqs::GateOp>& ops, int want_halves) {
    const int n = 14;
    const std::vector<hqs::LaunchPlan> L = hqs::plan_launches(n, hqs::kArithTC, ops, 11, 16, true);
    for (const hqs::LaunchPlan& l : L) {
        if (!l.umma) continue;
        const hqs::UmmaDesc& u = l.udesc;
        const int halves = u.d.nops == 1 ? 1 : 0;
        if (halves != want_halves) {
            std::printf("%s halves=%d expected %d FAIL\n", name, halves, want_halves);
            return 1;
        }
        std::vector<unsigned char> pool(l.pool_bytes + 64);
        hqs::write_umma_pool(u, ops.data() + l.first, pool.data());
        const unsigned char* gate = pool.data() + u.gate_off;
        const uint16_t* planes = reinterpret_cast<const uint16_t*>(gate);
        const int32_t* ecol = reinterpret_cast<const int32_t*>(gate + hqs::kUmmaGatePlaneBytes);
        const hqs::GateOp& g = ops[l.first + (size_t)u.tc_op];
        double worst = 0.0;
        for (int nn = 0; nn < 64; ++nn) {
            int ebmax = 0;
            for (int kk = 0; kk < 64; ++kk) ebmax = std::max(ebmax, biased_exponent(real_form(g, kk, nn)));
            if (ecol[nn] != ebmax) {
                std::printf("%s column %d exponent %d expected %d FAIL\n", name, nn, ecol[nn], ebmax);
                return 1;
            }
            for (int kk = 0; kk < 64; ++kk) {
                double v = 0.0;
                for (int j = 0; j < 6; ++j) {
                    const int row = halves ? 192 * (nn >> 5) + 32 * j + (nn & 31) : 64 * j + nn;
                    const size_t byte = (size_t)row * 128 + ((size_t)(((2 * kk) >> 4) ^ (row & 7)) << 4) + ((2 * kk) & 15);
                    v += std::ldexp(f16_value(planes[byte / 2]), -9 * j);
                }
                v = std::ldexp(v, ebmax - 1029);
                const double unit = std::ldexp(1.0, ebmax - 1074);
                worst = std::max(worst, std::fabs(v - real_form(g, kk, nn)) / unit);
            }
        }
        const bool ok = worst <= 0.5000001;
        std::printf("%s halves=%d max_units=%.3f %s\n", name, halves, worst, ok ? "ok" : "FAIL");
        return ok ? 0 : 1;
    }
    std::printf("%s no tensor-memory launch FAIL\n", name);
    return 1;
}

}  // namespace

int main() {
    // a dense five-qubit gate with entries of mixed magnitudes (a fixed
    // linear congruential sequence), then the same gate followed by a
    // diagonal one-qubit gate outside its targets
    hqs::GateOp g;
    g.k = 5;
    const int pos[5] = {1, 3, 6, 9, 12};
    for (int t = 0; t < 5; ++t) g.pos[t] = pos[t];
    uint64_t s = 12345;
    auto next = [&]() {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(s >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    };
    g.m.resize(32 * 32);
    for (size_t e = 0; e < g.m.size(); ++e) {
        const double sc = std::ldexp(1.0, -(int)(e % 7) * 3);
        g.m[e] = hqs::cplx(next() * sc, next() * sc);
    }
    hqs::GateOp dg;
    dg.k = 1;
    dg.diag = true;
    dg.pos[0] = 0;
    dg.m = {hqs::cplx(0.6, 0.8), hqs::cplx(0.0, -1.0)};
    int bad = 0;
    bad += check("dense", {g}, 1);
    bad += check("dense+diagonal", {g, dg}, 0);
    return bad;
}
