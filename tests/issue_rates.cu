// Issue-rate microbenchmark of the arithmetic the tracer step is built from: FP64 FMA,
// add and multiply, FP32 FMA, FP64<->FP32 conversions and FP64 division, each as 8
// independent chains per thread over 8 CTAs of 256 threads per SM.  Prints operations per
// clock per SM at the nominal 2.07 GHz (the design of the FP32-flux form rests on the
// ratio of these rates on GB300).
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x)                                                                       \
    do {                                                                            \
        cudaError_t e_ = (x);                                                       \
        if (e_ != cudaSuccess) {                                                    \
            printf("CUDA error %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
            return 1;                                                               \
        }                                                                           \
    } while (0)

template <int OP>
__global__ void k_rate(double *out, int iters, double a, double b)
{
    double x[8];
    float f[8];
    for (int u = 0; u < 8; u++) {
        x[u] = threadIdx.x * 1e-3 + u;
        f[u] = (float)x[u];
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (OP == 0) x[u] = fma(x[u], a, b);
            if (OP == 1) x[u] = __dadd_rn(x[u], b);
            if (OP == 2) x[u] = __dmul_rn(x[u], a);
            if (OP == 3) f[u] = fmaf(f[u], (float)a, (float)b);
            if (OP == 4) {   // FP64 -> FP32 -> FP64 and an add
                f[u] = __double2float_rn(x[u]);
                x[u] = (double)f[u] + b;
            }
            if (OP == 5) x[u] = b / x[u];
        }
    }
    double s = 0;
    for (int u = 0; u < 8; u++) s += x[u] + f[u];
    if (s == 12345.678) out[threadIdx.x] = s;
}

template <int OP>
int run(const char *name, int nsm)
{
    double *d;
    CK(cudaMalloc(&d, 1024 * sizeof(double)));
    const int blocks = nsm * 8, threads = 256, iters = OP == 5 ? 64 : 2048;
    k_rate<OP><<<blocks, threads>>>(d, 16, 1.0000001, 1e-9);
    CK(cudaDeviceSynchronize());
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    k_rate<OP><<<blocks, threads>>>(d, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    const double n = (double)blocks * threads * iters * 8;
    printf("%-32s %8.3f ms %10.1f Gop/s %8.2f op/clk/SM\n", name, ms, n / ms / 1e6, n / (ms * 1e-3) / nsm / 2.07e9);
    cudaFree(d);
    return 0;
}

int main()
{
    cudaDeviceProp p;
    CK(cudaGetDeviceProperties(&p, 0));
    printf("%s SMs=%d cc=%d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
    const int n = p.multiProcessorCount;
    int r = run<0>("DFMA", n) | run<1>("DADD", n) | run<2>("DMUL", n) | run<3>("FFMA", n) |
            run<4>("F2F d->f->d + DADD (per chain op)", n) | run<5>("DDIV (per division)", n);
    return r;
}
