// FP32-flux / FP64-state form of the tracer step (one grid, and the
// per-member data the batched ensemble kernel reads).
#pragma once

#include "gb_internal.h"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace gbgo {

struct Fp32Member {
    bool ready = false;
    void *impl = nullptr;   // owned device data, see tstep_fp32.cu
};

int fp32_member_init(Fp32Member *f, const Dims &d, const PhysParams &p, const Metrics &m,
                     const std::vector<double> &blob, const int32_t *k1_host, cudaStream_t s, std::string &msg);
void fp32_member_free(Fp32Member *f);
int fp32_member_upload(Fp32Member *f, const double *ts_cur, const double *ts_static, cudaStream_t s);
int fp32_member_set_top(Fp32Member *f, const double *top, cudaStream_t s);
int fp32_member_set_velocity(Fp32Member *f, const double *u, cudaStream_t s);
int fp32_member_step(Fp32Member *f, double *ts_buf[2], int *cur, double *rho, const double *ts_static, double *cost,
                     int32_t *icosd, unsigned long long *diag, int *slot, int nsteps, cudaStream_t s);
int fp32_member_export(Fp32Member *f, const double *ts_cur, double *rho, const double *ts_static, cudaStream_t s);

void count_launches(uint64_t n);

}  // namespace gbgo
