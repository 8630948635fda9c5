// GOLDSTEIN time-series diagnostics on the device-resident ocean (include/gb_timeseries.h):
//   diag2     src/goldstein/goldstein_diag.f90:10-71
//   diagopsi  src/goldstein/goldstein_diag.f90:350-411
//   records   src/goldstein/goldstein.f90:284-310 (formats 100, 110)
//
// The reference forms each regional sum, avn and avs as one left-to-right chain over the wet
// cells in its (k, j, i) loop order.  Here every chain is one device thread walking an ordered
// cell list built once per grid, with round-to-nearest intrinsics in the reference's operation
// order (compiled with -fmad=false as well), so each number is the reference's bit for bit.  A
// chain of n additions costs n dependent FP64 adds (~63 cycles each on GB300); the chains run
// side by side, one per (region, tracer), plus avn and avs.  The overturning streamfunctions
// take one thread per row (the i sums and the k recurrence in order), the extrema one thread
// in the reference's (j, k) scan order.
#include "gb_internal.h"
#include "../../include/gb_timeseries.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace gbgo;

struct gb_ts_handle {
    int device = 0;
    gb_go_dims dims{};
    int NI = 0, NJ = 0;
    double dphi = 0.0;
    long long ntot = 0, intot = 0;
    double vol[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int32_t jsf = 0, overdep = 0;
    // device
    int2 *cells = nullptr;        // region lists: (ts cell offset, j | k << 16), regions back to back
    int *roff = nullptr;          // region r's list: cells[roff[r], roff[r+1])
    int4 *all = nullptr;          // every wet cell in loop order: (ts cell offset, i, j, k)
    double *ds = nullptr, *dz = nullptr, *dza = nullptr, *cv = nullptr, *volv = nullptr;   // Fortran-indexed
    int32_t *basin = nullptr;     // ips, ipf, ias, iaf: 4 x (maxj + 1), Fortran-indexed rows
    double *opsi = nullptr;       // opsi, opsip, opsia: 3 x (maxj+1)(maxk+1)
    double *res = nullptr;        // 8 L sums, avn, avs, ext[4], iposa[2]
    std::vector<double> res_host;
    std::string last_error;
};

static int tsfail(gb_ts_handle *h, int code, const std::string &msg)
{
    if (h) h->last_error = msg;
    return code;
}

#define TS_TRY(h, call)                                                                                 \
    do {                                                                                                \
        cudaError_t _x = (call);                                                                        \
        if (_x != cudaSuccess)                                                                          \
            return tsfail(h, _x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA,                \
                          std::string(#call) + ": " + cudaGetErrorString(_x));                          \
    } while (0)

namespace {

// diag2's chains: thread t < 8 L sums region t % 8 of tracer t / 8; thread 8 L forms avn, thread
// 8 L + 1 avs (goldstein_diag.f90:22-69).
__global__ void k_ts_chains(const int2 *__restrict__ cells, const int *__restrict__ roff, const int4 *__restrict__ all,
                            int nall, const double *__restrict__ ts, const double *__restrict__ rho,
                            const double *__restrict__ u, int L, int maxi, int maxj, int maxk, int NI, int NJ,
                            double dphi, const double *__restrict__ ds, const double *__restrict__ dz,
                            const double *__restrict__ dza, const double *__restrict__ vol, long long ntot,
                            long long intot, double *__restrict__ res)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 8 * L) {
        const int r = t % 8, l = t / 8;
        double s = 0.0;
        for (int e = roff[r]; e < roff[r + 1]; ++e) {
            const int2 c = cells[e];
            const int j = c.y & 0xffff, k = c.y >> 16;
            s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(ts[(size_t)c.x * L + l], dphi), ds[j]), dz[k]));
        }
        res[r + 8 * l] = vol[r] != 0.0 ? __ddiv_rn(s, vol[r]) : s;
    } else if (t == 8 * L) {
        double s = 0.0;
        for (int e = 0; e < nall; ++e) {
            const int4 c = all[e];
            if (c.w < maxk) {
                const size_t o = (size_t)c.y + (size_t)NI * ((size_t)c.z + (size_t)NJ * (size_t)c.w);
                s = __dadd_rn(s, __ddiv_rn(fabs(__dsub_rn(rho[o], rho[o + (size_t)NI * NJ])), dza[c.w]));
            }
        }
        res[8 * L] = __ddiv_rn(s, (double)intot);
    } else if (t == 8 * L + 1) {
        double s = 0.0;
        for (int e = 0; e < nall; ++e) {
            const int4 c = all[e];
            const size_t o = 3 * ((size_t)c.y + (size_t)(maxi + 1) * ((size_t)c.z + (size_t)(maxj + 1) * (size_t)(c.w - 1)));
            const double u1 = u[o], u2 = u[o + 1];
            s = __dadd_rn(__dadd_rn(s, __dmul_rn(u1, u1)), __dmul_rn(u2, u2));
        }
        res[8 * L + 1] = __dsqrt_rn(__ddiv_rn(s, (double)ntot));
    }
}

// diagopsi's streamfunctions, one thread per row j = 1..maxj-1 (goldstein_diag.f90:362-400):
// ou(j,k) = the sum over the basin's longitudes of cv(j) * u(2,i,j,k) * dphi, left to right;
// psi(j,k) = psi(j,k-1) - dz(k) * ou(j,k).  Arrays (0:maxj, 0:maxk), zero where not formed.
__global__ void k_ts_opsi(const double *__restrict__ u, int maxi, int maxj, int maxk, double dphi,
                          const double *__restrict__ cv, const double *__restrict__ dz, const int32_t *__restrict__ basin,
                          int jsf, double *__restrict__ opsi)
{
    const int nj = maxj + 1;
    const size_t plane = (size_t)nj * (maxk + 1);
    double *op = opsi, *opp = opsi + plane, *opa = opsi + 2 * plane;
    const int32_t *ips = basin, *ipf = basin + nj, *ias = basin + 2 * nj, *iaf = basin + 3 * nj;
    auto U2 = [&](int i, int j, int k) {
        return u[1 + 3 * ((size_t)i + (size_t)(maxi + 1) * ((size_t)j + (size_t)(maxj + 1) * (size_t)(k - 1)))];
    };
    for (int j = 1 + blockIdx.x * blockDim.x + threadIdx.x; j <= maxj - 1; j += gridDim.x * blockDim.x) {
        const double cj = cv[j];
        auto term = [&](int i, int k) { return __dmul_rn(__dmul_rn(cj, U2(i, j, k)), dphi); };
        for (int k = 1; k <= maxk - 1; ++k) {
            double ou = 0.0;
            for (int i = 1; i <= maxi; ++i) ou = __dadd_rn(ou, term(i, k));
            op[j + (size_t)nj * k] = __dsub_rn(op[j + (size_t)nj * (k - 1)], __dmul_rn(dz[k], ou));
        }
        if (j < jsf + 1) continue;
        for (int k = 1; k <= maxk - 1; ++k) {
            double ou = 0.0;
            for (int i = ips[j]; i <= ipf[j]; ++i) ou = __dadd_rn(ou, term(i, k));
            opp[j + (size_t)nj * k] = __dsub_rn(opp[j + (size_t)nj * (k - 1)], __dmul_rn(dz[k], ou));
        }
        for (int k = 1; k <= maxk - 1; ++k) {
            double ou = 0.0;
            if (ias[j] > iaf[j]) {   // the Atlantic wraps through i = maxi
                for (int i = ias[j]; i <= maxi; ++i) ou = __dadd_rn(ou, term(i, k));
                for (int i = 1; i <= iaf[j]; ++i) ou = __dadd_rn(ou, term(i, k));
            } else {
                for (int i = ias[j]; i <= iaf[j]; ++i) ou = __dadd_rn(ou, term(i, k));
            }
            opa[j + (size_t)nj * k] = __dsub_rn(opa[j + (size_t)nj * (k - 1)], __dmul_rn(dz[k], ou));
        }
    }
}

// The Pacific and Atlantic extrema in the reference's scan order (goldstein_diag.f90:369-409).
__global__ void k_ts_extrema(const double *__restrict__ opsi, int maxj, int maxk, int jsf, int overdep, double *res)
{
    const int nj = maxj + 1;
    const size_t plane = (size_t)nj * (maxk + 1);
    const double *opp = opsi + plane, *opa = opsi + 2 * plane;
    double ominp = 0.0, omaxp = 0.0, omina = 0.0, omaxa = 0.0;
    int ja = 0, ka = 0;
    for (int j = jsf + 1; j <= maxj - 1; ++j)
        for (int k = 1; k <= maxk - 1; ++k) {
            const double v = opp[j + (size_t)nj * k];
            if (v < ominp && k <= overdep) ominp = v;
            if (v > omaxp && k <= overdep) omaxp = v;
        }
    for (int j = jsf + 1; j <= maxj - 1; ++j)
        for (int k = 1; k <= maxk - 1; ++k) {
            const double v = opa[j + (size_t)nj * k];
            if (v < omina && k <= overdep) omina = v;
            if (v > omaxa && k <= overdep) {
                omaxa = v;
                ja = j;
                ka = k;
            }
        }
    res[0] = ominp;
    res[1] = omaxp;
    res[2] = omina;
    res[3] = omaxa;
    res[4] = (double)ja;
    res[5] = (double)ka;
}

// Fortran Ew.d output with w = 14, d = 6 (gfortran): 0.dddddd with the exponent as E+dd, or as
// +ddd without the E for exponents beyond two digits, right-justified in 14 characters.
void put_e14_6(char *out, double v)
{
    char body[32];
    if (std::isnan(v)) {
        std::snprintf(body, sizeof body, "NaN");
    } else if (std::isinf(v)) {
        std::snprintf(body, sizeof body, "%sInfinity", v < 0 ? "-" : "");
    } else if (v == 0.0) {
        std::snprintf(body, sizeof body, "%s0.000000E+00", std::signbit(v) ? "-" : "");
    } else {
        char b[40];
        std::snprintf(b, sizeof b, "%.5E", std::fabs(v));   // d.dddddE+xx, 6 significant digits
        const int e = std::atoi(std::strchr(b, 'E') + 1) + 1;
        char digits[7] = {b[0], b[2], b[3], b[4], b[5], b[6], 0};
        const char *sg = v < 0 ? "-" : "";
        if (e >= -99 && e <= 99)
            std::snprintf(body, sizeof body, "%s0.%sE%c%02d", sg, digits, e < 0 ? '-' : '+', e < 0 ? -e : e);
        else
            std::snprintf(body, sizeof body, "%s0.%s%c%03d", sg, digits, e < 0 ? '-' : '+', e < 0 ? -e : e);
    }
    std::snprintf(out, 15, "%14s", body);
}

}  // namespace

extern "C" int gb_ts_create(const gb_go_dims *dims, const gb_go_grid *grid, const gb_ts_basins *b, int device,
                            gb_ts_handle **out)
{
    if (!out) return GB_GO_EINVAL;
    *out = nullptr;
    if (!dims || !grid || !b || !grid->k1 || !grid->ds || !grid->dz || !grid->dza || !grid->cv || !b->ips || !b->ipf ||
        !b->ias || !b->iaf)
        return GB_GO_EINVAL;
    const int maxi = dims->maxi, maxj = dims->maxj, maxk = dims->maxk, L = dims->maxl;
    if (maxi < 1 || maxj < 2 || maxk < 1 || L < 1 || maxi > 65535 || maxj > 65535 || maxk > 32767) return GB_GO_EINVAL;
    gb_ts_handle *h = new gb_ts_handle();
    if (b->jsf < 0 || b->jsf > maxj || b->overdep < 0 || b->overdep > maxk) {
        delete h;
        return GB_GO_EINVAL;
    }
    for (int j = 0; j < maxj; ++j)
        for (const int32_t *a : {b->ips, b->ipf, b->ias, b->iaf})
            if (a[j] < 0 || a[j] > maxi) {
                delete h;
                return GB_GO_EINVAL;
            }
    if (device < 0) cudaGetDevice(&h->device);
    else h->device = device;
    h->dims = *dims;
    h->NI = maxi + 2;
    h->NJ = maxj + 2;
    h->dphi = grid->dphi;
    h->jsf = b->jsf;
    h->overdep = b->overdep;
    const int NI = h->NI, NJ = h->NJ;
    // region lists and volumes in diag2's loop order (goldstein_diag.f90:22-44)
    std::vector<std::vector<int2>> reg(8);
    std::vector<int4> all;
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                if (k < grid->k1[i + (size_t)NI * j]) continue;
                const int ndep = (2 * k - 1) / maxk;
                int mo;
                const int ips = b->ips[j - 1], ipf = b->ipf[j - 1], ias = b->ias[j - 1], iaf = b->iaf[j - 1];
                if (j <= b->jsf) mo = 4;
                else if (i >= ips && i <= ipf) mo = 1;
                else if ((i >= ias && i <= iaf) || (iaf <= ias && (i <= iaf || ias <= i))) mo = 2;
                else mo = 3;
                const int r = mo + 4 * ndep - 1;
                const int c = i + NI * (j + NJ * k);
                reg[r].push_back(make_int2(c, j | (k << 16)));
                all.push_back(make_int4(c, i, j, k));
                h->vol[r] = h->vol[r] + grid->dphi * grid->ds[j - 1] * grid->dz[k - 1];
            }
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i) {
            const int k1 = grid->k1[i + (size_t)NI * j];
            if (k1 <= maxk) {
                h->ntot += maxk - k1 + 1;
                h->intot += maxk - k1;
            }
        }
    std::vector<int2> cells;
    std::vector<int> roff(9, 0);
    for (int r = 0; r < 8; ++r) {
        roff[r] = (int)cells.size();
        cells.insert(cells.end(), reg[r].begin(), reg[r].end());
    }
    roff[8] = (int)cells.size();
    // Fortran-indexed metrics and basin rows
    std::vector<double> ds(maxj + 2, 0.0), dz(maxk + 2, 0.0), dza(maxk + 2, 0.0), cv(maxj + 2, 0.0);
    for (int j = 1; j <= maxj; ++j) ds[j] = grid->ds[j - 1];
    for (int j = 0; j <= maxj; ++j) cv[j] = grid->cv[j];
    for (int k = 1; k <= maxk; ++k) {
        dz[k] = grid->dz[k - 1];
        dza[k] = grid->dza[k - 1];
    }
    std::vector<int32_t> basin(4 * (size_t)(maxj + 1), 0);
    for (int j = 1; j <= maxj; ++j) {
        basin[j] = b->ips[j - 1];
        basin[(maxj + 1) + j] = b->ipf[j - 1];
        basin[2 * (maxj + 1) + j] = b->ias[j - 1];
        basin[3 * (maxj + 1) + j] = b->iaf[j - 1];
    }
    cudaError_t x = cudaSetDevice(h->device);
    auto up = [&](auto **dst, const auto &v) {
        using T = typename std::remove_reference<decltype(v[0])>::type;
        if (x == cudaSuccess) x = cudaMalloc((void **)dst, std::max<size_t>(1, v.size()) * sizeof(T));
        if (x == cudaSuccess && !v.empty()) x = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    };
    up(&h->cells, cells);
    up(&h->roff, roff);
    up(&h->all, all);
    up(&h->ds, ds);
    up(&h->dz, dz);
    up(&h->dza, dza);
    up(&h->cv, cv);
    up(&h->basin, basin);
    std::vector<double> volv(h->vol, h->vol + 8);
    up(&h->volv, volv);
    const size_t plane = (size_t)(maxj + 1) * (maxk + 1);
    if (x == cudaSuccess) x = cudaMalloc((void **)&h->opsi, 3 * plane * sizeof(double));
    h->res_host.assign(8 * (size_t)L + 8, 0.0);
    if (x == cudaSuccess) x = cudaMalloc((void **)&h->res, h->res_host.size() * sizeof(double));
    if (x != cudaSuccess) {
        gb_ts_destroy(h);
        return x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA;
    }
    *out = h;
    return GB_GO_OK;
}

extern "C" void gb_ts_destroy(gb_ts_handle *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    cudaFree(h->cells);
    cudaFree(h->roff);
    cudaFree(h->all);
    cudaFree(h->ds);
    cudaFree(h->dz);
    cudaFree(h->dza);
    cudaFree(h->cv);
    cudaFree(h->basin);
    cudaFree(h->volv);
    cudaFree(h->opsi);
    cudaFree(h->res);
    delete h;
}

extern "C" int gb_ts_diagnose(gb_ts_handle *h, gb_go_handle *ocean, double *sums, double *avn, double *avs, double *ext,
                              int32_t *iposa, double *opsi, double *opsip, double *opsia)
{
    gbgo::TraceRange tr_("ts_diagnose");
    if (!h || !ocean) return GB_GO_EINVAL;
    OceanState o{};
    if (ocean_state(ocean, &o) != GB_GO_OK) return tsfail(h, GB_GO_EINVAL, "bad ocean handle");
    const gb_go_dims &d = h->dims;
    if (o.d.maxi != d.maxi || o.d.maxj != d.maxj || o.d.maxk != d.maxk || o.d.L != d.maxl)
        return tsfail(h, GB_GO_EINVAL, "ocean handle of another shape");
    if (o.device != h->device) return tsfail(h, GB_GO_EINVAL, "ocean handle on another device");
    if (!o.state_ready) return tsfail(h, GB_GO_ENOTREADY, "ocean state not uploaded");
    TS_TRY(h, cudaSetDevice(h->device));
    // the split-precision form exports its state (Fortran layout) and rho first
    if (const int rr = ocean_refresh_rho(ocean))
        return tsfail(h, rr, std::string("state export failed: ") + gb_go_last_error(ocean));
    cudaStream_t s = (cudaStream_t)o.stream;
    const double *ts = o.steps_since_upload > 0 ? o.ts_buf[o.cur] : o.ts_static;
    const int L = d.maxl;
    const size_t plane = (size_t)(d.maxj + 1) * (d.maxk + 1);
    TS_TRY(h, cudaMemsetAsync(h->opsi, 0, 3 * plane * sizeof(double), s));
    const int nth = 8 * L + 2;
    k_ts_chains<<<(nth + 63) / 64, 64, 0, s>>>(h->cells, h->roff, h->all, (int)h->ntot, ts, o.rho, o.u, L, d.maxi, d.maxj,
                                               d.maxk, h->NI, h->NJ, h->dphi, h->ds, h->dz, h->dza, h->volv, h->ntot,
                                               h->intot, h->res);
    k_ts_opsi<<<std::max(1, (d.maxj + 63) / 64), 64, 0, s>>>(o.u, d.maxi, d.maxj, d.maxk, h->dphi, h->cv, h->dz, h->basin,
                                                             h->jsf, h->opsi);
    k_ts_extrema<<<1, 1, 0, s>>>(h->opsi, d.maxj, d.maxk, h->jsf, h->overdep, h->res + 8 * L + 2);
    count_launches(3);
    TS_TRY(h, cudaGetLastError());
    TS_TRY(h, cudaMemcpyAsync(h->res_host.data(), h->res, h->res_host.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (opsi) TS_TRY(h, cudaMemcpyAsync(opsi, h->opsi, plane * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (opsip) TS_TRY(h, cudaMemcpyAsync(opsip, h->opsi + plane, plane * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (opsia) TS_TRY(h, cudaMemcpyAsync(opsia, h->opsi + 2 * plane, plane * sizeof(double), cudaMemcpyDeviceToHost, s));
    TS_TRY(h, cudaStreamSynchronize(s));
    const double *r = h->res_host.data();
    if (sums) std::memcpy(sums, r, 8 * (size_t)L * sizeof(double));
    if (avn) *avn = r[8 * L];
    if (avs) *avs = r[8 * L + 1];
    if (ext) std::memcpy(ext, r + 8 * L + 2, 4 * sizeof(double));
    if (iposa) {
        iposa[0] = (int32_t)r[8 * L + 6];
        iposa[1] = (int32_t)r[8 * L + 7];
    }
    return GB_GO_OK;
}

extern "C" int gb_ts_format(double time, int32_t maxl, const double *sums, double avn, double avs, const double *ext,
                            const int32_t *iposa, double opsisc, char *t_line, char *s_line, char *opsit_line, int32_t len)
{
    if (!sums || !ext || !iposa || maxl < 2 || len < 160) return GB_GO_EINVAL;
    auto row = [&](char *out, const double *v8) {
        char *p = out;
        put_e14_6(p, time);
        p += 14;
        for (int n = 0; n < 8; ++n, p += 14) put_e14_6(p, v8[n]);
        put_e14_6(p, avn);
        p += 14;
        put_e14_6(p, avs);
        p += 14;
        *p++ = '\n';
        *p = 0;
    };
    if (t_line) row(t_line, sums);
    if (s_line) row(s_line, sums + 8);
    if (opsit_line) {
        char *p = opsit_line;
        put_e14_6(p, time);
        p += 14;
        for (int n = 0; n < 4; ++n, p += 14) put_e14_6(p, ext[n] * opsisc);
        std::snprintf(p, 12, "%5d%5d\n", (int)iposa[0], (int)iposa[1]);
    }
    return GB_GO_OK;
}

extern "C" const char *gb_ts_last_error(const gb_ts_handle *h) { return h ? h->last_error.c_str() : ""; }
