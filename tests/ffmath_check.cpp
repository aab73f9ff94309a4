// Host build of quasi_gb300/csrc/ffmath.cuh: the device intrinsics it uses are IEEE
// round-to-nearest float operations, so mapping them to host float arithmetic (compiled with
// -ffp-contract=off) reproduces the device results. Prints the worst relative error of each
// double-float operation against long double over random inputs.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <random>

#include <cuda_runtime.h>

inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __fsqrt_rn(float a) { return std::sqrt(a); }
inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
#include "../quasi_gb300/csrc/ffmath.cuh"

using quasi::ff;
static long double val(ff a) { return (long double)a.hi + (long double)a.lo; }

int main() {
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(-2.0, 2.0), P(1e-3, 4.0), R01(0.0, 1.0);
    long double e_add = 0, e_addf = 0, e_mul = 0, e_div = 0, e_sqrt = 0, e_sin = 0, e_cos = 0, e_dotsub = 0;
    std::uniform_real_distribution<double> LogD(-12.0, 0.0);
    auto mk = [&](double d) { ff x; x.hi = (float)d; x.lo = (float)(d - (double)x.hi); return x; };
    for (int i = 0; i < 200000; ++i) {
        const ff a = mk(U(rng)), b = mk(U(rng)), p = mk(P(rng));
        const long double A = val(a), B = val(b), Pv = val(p);
        auto rel = [](long double got, long double want) {
            return fabsl(got - want) / fmaxl(fabsl(want), 1e-30L);
        };
        const long double scale = fmaxl(fabsl(A), fabsl(B));
        e_add = fmaxl(e_add, fabsl(val(quasi::ff_add(a, b)) - (A + B)) / fmaxl(scale, 1e-30L));
        e_addf = fmaxl(e_addf, fabsl(val(quasi::ff_add_fast(a, b)) - (A + B)) / fmaxl(fabsl(A) + fabsl(B), 1e-30L));
        e_mul = fmaxl(e_mul, rel(val(quasi::ff_mul(a, b)), A * B));
        e_div = fmaxl(e_div, rel(val(quasi::ff_div(a, p)), A / Pv));
        e_sqrt = fmaxl(e_sqrt, rel(val(quasi::ff_sqrt(p)), sqrtl(Pv)));
        const float x = (float)(2.0 * R01(rng));
        ff s, c;
        quasi::ff_sincospi(x, s, c);
        const long double pi = 3.141592653589793238462643383279502884L;
        e_sin = fmaxl(e_sin, fabsl(val(s) - sinl(pi * (long double)x)));
        e_cos = fmaxl(e_cos, fabsl(val(c) - cosl(pi * (long double)x)));
        // a . b - c for a unit a and a b nearly orthogonal to it (a grazing cosine): beyond the
        // final rounding to float (2^-24 of the result) the error must stay near 2^-48 of the
        // terms' magnitudes, however small the result
        {
            const double ux = U(rng), uy = U(rng), uz = U(rng), ul = std::sqrt(ux * ux + uy * uy + uz * uz) + 1e-9;
            const double nx = ux / ul, ny = uy / ul, nz = uz / ul;
            double tx = U(rng), ty = U(rng), tz = U(rng);
            const double tn = tx * nx + ty * ny + tz * nz, delta = std::pow(10.0, LogD(rng));
            tx += (delta - tn) * nx;
            ty += (delta - tn) * ny;
            tz += (delta - tn) * nz;
            const quasi::ff3 na{mk(nx), mk(ny), mk(nz)}, tb{mk(tx), mk(ty), mk(tz)};
            const float cc = (i & 1) ? 1e-4f : 0.0f;
            const long double terms[3] = {val(na.x) * val(tb.x), val(na.y) * val(tb.y), val(na.z) * val(tb.z)};
            const long double want = terms[0] + terms[1] + terms[2] - (long double)cc;
            const long double mag = fabsl(terms[0]) + fabsl(terms[1]) + fabsl(terms[2]) + fabsl((long double)cc);
            const long double got = quasi::ff3_dot_sub(na, tb, cc);
            const long double beyond = fabsl(got - want) - 0x1p-24L * fabsl(want);
            e_dotsub = fmaxl(e_dotsub, fmaxl(beyond, 0.0L) / mag);
        }
    }
    std::printf("add %.3Le\naddf %.3Le\nmul %.3Le\ndiv %.3Le\nsqrt %.3Le\nsin %.3Le\ncos %.3Le\ndotsub %.3Le\n", e_add,
                e_addf, e_mul, e_div, e_sqrt, e_sin, e_cos, e_dotsub);
    return 0;
}
