// Checks that div_rn_recip (co_column.cuh) returns the IEEE quotient __ddiv_rn(a, b) bit
// for bit: random numerators of both signs over a wide exponent range, positive divisors
// as the convective adjustment makes them (sums of layer thicknesses), and edge cases
// (zero, exact quotients, powers of two).  Prints the number of mismatches and exits 1 if
// there is any.
#include "co_column.cuh"

#include <cstdio>
#include <cstdint>

using namespace gbgo;

__device__ __forceinline__ uint64_t mix(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

__device__ double make(uint64_t r, int emin, int span, bool sign)
{
    const uint64_t mant = r & 0xfffffffffffffULL;
    const int e = emin + (int)((r >> 52) % (uint64_t)span);
    const uint64_t s = sign ? ((r >> 63) << 63) : 0;
    return __longlong_as_double((long long)(s | ((uint64_t)(e + 1023) << 52) | mant));
}

__global__ void k_check(uint64_t n, uint64_t seed, unsigned long long *bad, unsigned long long *fast)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r1 = mix(seed + 2 * i), r2 = mix(seed + 2 * i + 1);
        double a = make(r1, -40, 80, true);
        double b = make(r2, -10, 24, false);
        switch (i % 16) {
        case 0: a = 0.0; break;
        case 1: a = b * (double)(int)(r1 % 1000); break;                    // exact quotients
        case 2: b = __longlong_as_double((long long)(((r2 % 40) + 1003) << 52)); break;   // powers of two
        case 3: a = b * __longlong_as_double((long long)(((r1 % 40) + 1003) << 52)); break;
        case 4: b = (double)(1 + r2 % 64) * 0.125; break;                   // few-bit divisors
        default: break;
        }
        const double y = __drcp_rn(b);
        const double q = div_rn_recip(a, b, y);
        const double ref = __ddiv_rn(a, b);
        if (__double_as_longlong(q) != __double_as_longlong(ref)) atomicAdd(bad, 1ull);
    }
    (void)fast;
}

int main()
{
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    const uint64_t n = 1ull << 26;
    for (uint64_t seed = 1; seed <= 4; ++seed) k_check<<<2048, 256>>>(n, seed * 0x9e3779b97f4a7c15ULL, d, d + 1);
    unsigned long long h[2] = {0, 0};
    if (cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
    printf("checked %llu quotients, mismatches %llu\n", (unsigned long long)(4 * n), h[0]);
    cudaFree(d);
    return h[0] ? 1 : 0;
}
