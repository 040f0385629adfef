// Window probe for tests/test_gpu_windows.py: the largest distance, in
// half-ulps of the rounded result, between each faithful helper's
// float-float value r + d (mhd-gpu_gb300/csrc/mhd_math.cuh) and the C path's
// double value of the same expression, over seeded random operands (half of
// them in realistic ranges, half with random mantissas over wide exponent
// ranges).  The near-boundary windows (kKPressure, kKSlope, kKSpeed, kKCfl)
// must be wider than these distances, or a value outside a window could
// round differently from the C path.
//
//   window_probe <samples> <seed>
// prints one line per helper: "<name> <samples> <log2 of the largest
// distance in half-ulps> <K>".
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "../mhd-gpu_gb300/csrc/mhd_math.cuh"

using namespace mhd;

namespace {

__device__ unsigned g_max[4];             // float bits of the largest distance (half-ulps)
__device__ unsigned long long g_count[4];

__device__ __forceinline__ unsigned mix(unsigned x)
{
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float uniform(unsigned &s)
{
    s = mix(s + 0x9e3779b9U);
    return (float)(s >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float normal(unsigned &s)
{
    const float a = fmaxf(uniform(s), 1e-7f), b = uniform(s);
    return sqrtf(-2.0f * logf(a)) * cospif(2.0f * b);
}
// a float with a random mantissa and an exponent in [lo, hi)
__device__ __forceinline__ float wide(unsigned &s, int lo, int hi)
{
    s = mix(s + 0x85ebca6bU);
    const float m = 1.0f + (float)(s >> 9) * (1.0f / 8388608.0f);
    return ldexpf(m, lo + (int)((float)(hi - lo) * uniform(s)));
}

// the distance of r + d from the exact double value, in half-ulps of r
__device__ void record(int h, float r, float d, double exact)
{
    const float ar = fabsf(r);
    const double half = 0.5 * (double)(__uint_as_float(__float_as_uint(ar) + 1u) - ar);
    const double dist = fabs(((double)r + (double)d) - exact) / half;
    atomicMax(&g_max[h], __float_as_uint((float)dist));
    atomicAdd(&g_count[h], 1ull);
}

__global__ void probe(unsigned long long n, unsigned seed)
{
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned s = mix((unsigned)i * 2654435761U ^ seed ^ (unsigned)(i >> 32));
        const bool w = (i & 1) != 0;
        {   // total pressure (E - q/2)(gamma - 1) + (2 - gamma) B2/2, mhdflux.c:28
            const float e = w ? wide(s, -4, 8) : 1.5f + 0.5f * normal(s);
            float q = w ? wide(s, -8, 6) : fabsf(normal(s)) * 0.5f;
            const float b2 = w ? wide(s, -8, 8) : fabsf(normal(s)) * 2.0f;
            if (0.5f * q >= e) q = e;
            float d;
            bool neg;
            const float r = total_pressure_rd(e, q, b2, d, neg);
            const double a = mhd::dsub((double)e, mhd::dmul((double)q, 0.5));
            const double exact = mhd::dadd(mhd::dmul(a, (double)kGammaM1), mhd::dmul((double)kTwoMGammaHalf, (double)b2));
            if (!neg && r > 0.0f) record(0, r, d, exact);
        }
        {   // van Leer quotient XY/(X+Y), tvd1.c:78
            float X, Y;
            if (w) {
                X = wide(s, -30, 10);
                Y = wide(s, -30, 10);
            } else {
                X = fabsf(normal(s)) * exp10f(-6.0f + 7.0f * uniform(s));
                Y = fabsf(X * (1.0f + 0.5f * normal(s))) + 1e-3f * fabsf(normal(s));
            }
            if (uniform(s) < 0.5f) { X = -X; Y = -Y; }
            float d, ph;
            const float q = Faithful::slope_rd(X, Y, d, ph);
            if (ph > 0.0f && isfinite(q) && q != 0.0f) {
                const double exact = mhd::ddiv(mhd::dadd((double)ph, (double)ffma(X, Y, -ph)), (double)fadd(X, Y));
                record(1, q, d, exact);
            }
        }
        {   // fast speed x + sqrt(a), mhdflux.c:45 (an exact root is not flagged)
            const float x = w ? wide(s, -12, 4) : fabsf(normal(s)) * (uniform(s) < 0.5f ? 0.1f : 1.0f);
            const float a = w ? wide(s, -20, 12) : fabsf(normal(s)) * 3.0f;
            float d, e0;
            const float r = Faithful::speed_rd(x, a, d, e0);
            if (a > 0.0f && e0 != 0.0f) record(2, r, d, mhd::dadd((double)x, mhd::dsqrt((double)a)));
        }
        {   // CFL speed v + sqrt(|2 B2 + gamma p| / rho), calcfl.c:54
            const float v = w ? wide(s, -12, 4) : fabsf(normal(s)) * 0.5f;
            const float b2 = w ? wide(s, -12, 6) : fabsf(normal(s)) * 2.0f;
            const float rho = w ? wide(s, -4, 4) : 0.5f + 1.5f * uniform(s);
            const float p = w ? wide(s, -8, 6) : 0.1f + 5.0f * uniform(s);
            const float gp = fmul(kGamma, p);
            float d;
            const float r = cfl_tail_rd(v, b2, gp, rho, true, Faithful::recip(rho), d);
            const double exact =
                mhd::dadd((double)v, mhd::dsqrt(mhd::ddiv(fabs(mhd::dadd(mhd::dmul((double)b2, 2.0), (double)gp)), (double)rho)));
            record(3, r, d, exact);
        }
    }
}

}  // namespace

int main(int argc, char **argv)
{
    const unsigned long long n = argc > 1 ? strtoull(argv[1], nullptr, 10) : (1ull << 24);
    const unsigned seed = argc > 2 ? (unsigned)strtoul(argv[2], nullptr, 10) : 777u;
    probe<<<152 * 8, 256>>>(n, seed);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        printf("cuda error %s\n", cudaGetErrorString(e));
        return 1;
    }
    unsigned mx[4];
    unsigned long long cnt[4];
    cudaMemcpyFromSymbol(mx, g_max, sizeof mx);
    cudaMemcpyFromSymbol(cnt, g_count, sizeof cnt);
    const char *names[4] = {"pressure", "slope", "speed", "cfl"};
    const int ks[4] = {kKPressure, kKSlope, kKSpeed, kKCfl};
    for (int h = 0; h < 4; ++h) {
        float m;
        memcpy(&m, &mx[h], sizeof m);
        printf("%s %llu %.3f %d\n", names[h], cnt[h], m > 0.0f ? log2f(m) : -1000.0f, ks[h]);
    }
    return 0;
}
