// GOLDSTEIN restart files of a device-resident ocean: outm_netcdf / inm_netcdf
// (src/goldstein/goldstein_data.f90:10-354) over a netCDF classic-format codec of its own.
//
// netCDF classic format (Unidata's published specification): "CDF" + version byte (1: 32-bit
// offsets, 2: 64-bit), numrecs, then the dimension, global-attribute and variable lists; each
// list is ABSENT (two zero words) or a tag (0x0A dimensions, 0x0B variables, 0x0C attributes)
// and a count.  Names are a length and the bytes padded with NUL to 4; values are big-endian
// and padded to 4.  A variable entry is name, ndims, dimids (slowest first), its attribute
// list, type, vsize (its data size padded to 4) and begin (the file offset of its data).  The
// netCDF library places the data of the first variable right after the header and each next
// one at begin + vsize, which the writer does as well.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gb_internal.h"
#include "gb_restart.h"

namespace {

using namespace gbgo;

thread_local std::string g_err;

int rs_fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

enum NcType { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
constexpr uint32_t kTagDim = 0x0A, kTagVar = 0x0B, kTagAtt = 0x0C;

int type_size(int t)
{
    switch (t) {
    case NC_BYTE: case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT: case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
    default: return 0;
    }
}

size_t pad4(size_t n) { return (n + 3) & ~(size_t)3; }

void put_be(std::vector<uint8_t> &b, uint64_t v, int nbytes)
{
    for (int s = nbytes - 1; s >= 0; --s) b.push_back((uint8_t)(v >> (8 * s)));
}

void put_name(std::vector<uint8_t> &b, const std::string &s)
{
    put_be(b, s.size(), 4);
    b.insert(b.end(), s.begin(), s.end());
    while (b.size() % 4) b.push_back(0);
}

void store_be(uint8_t *p, uint64_t v, int nbytes)
{
    for (int s = 0; s < nbytes; ++s) p[s] = (uint8_t)(v >> (8 * (nbytes - 1 - s)));
}

uint64_t load_be(const uint8_t *p, int nbytes)
{
    uint64_t v = 0;
    for (int s = 0; s < nbytes; ++s) v = (v << 8) | p[s];
    return v;
}

// ---------------------------------------------------------------- writer: file layout
struct NcVar {
    std::string name;
    int type;
    std::vector<int> dimids;   // slowest first
    std::vector<std::pair<std::string, std::string>> text_atts;
    size_t nelems = 0;
    size_t begin = 0;
    size_t vsize() const { return pad4(nelems * (size_t)type_size(type)); }
};

struct NcLayout {
    std::vector<std::pair<std::string, size_t>> dims;
    std::vector<NcVar> vars;
    int version = 1;
    size_t header_bytes = 0, total_bytes = 0;

    std::vector<uint8_t> header() const
    {
        std::vector<uint8_t> b = {'C', 'D', 'F', (uint8_t)version};
        put_be(b, 0, 4);   // numrecs: no record dimension
        put_be(b, dims.empty() ? 0 : kTagDim, 4);
        put_be(b, dims.size(), 4);
        for (const auto &d : dims) {
            put_name(b, d.first);
            put_be(b, d.second, 4);
        }
        put_be(b, 0, 4);   // no global attributes
        put_be(b, 0, 4);
        put_be(b, vars.empty() ? 0 : kTagVar, 4);
        put_be(b, vars.size(), 4);
        for (const auto &v : vars) {
            put_name(b, v.name);
            put_be(b, v.dimids.size(), 4);
            for (int id : v.dimids) put_be(b, (uint64_t)id, 4);
            put_be(b, v.text_atts.empty() ? 0 : kTagAtt, 4);
            put_be(b, v.text_atts.size(), 4);
            for (const auto &a : v.text_atts) {
                put_name(b, a.first);
                put_be(b, NC_CHAR, 4);
                put_name(b, a.second);   // nelems + characters padded to 4: the same encoding
            }
            put_be(b, v.type, 4);
            const size_t vs = v.vsize();
            put_be(b, vs > 0xFFFFFFFCull ? 0xFFFFFFFFull : vs, 4);
            put_be(b, v.begin, version == 1 ? 4 : 8);
        }
        return b;
    }

    void place()
    {
        for (version = 1; version <= 2; ++version) {
            header_bytes = header().size();
            size_t off = header_bytes;
            for (auto &v : vars) {
                v.begin = off;
                off += v.vsize();
            }
            total_bytes = off;
            const size_t last_begin = vars.empty() ? 0 : vars.back().begin;
            if (last_begin <= 0x7FFFFFFFull) break;   // CDF-1 offsets are signed 32-bit
        }
    }

    const NcVar &var(const char *name) const
    {
        for (const auto &v : vars)
            if (v.name == name) return v;
        return vars.front();
    }
};

NcLayout goldstein_layout(int maxi, int maxj, int maxk, int gui)
{
    NcLayout L;
    L.dims = {{"nrecs", 1}, {"longitude", (size_t)maxi}, {"latitude", (size_t)maxj}, {"depth", (size_t)maxk}};
    const size_t n3 = (size_t)maxi * maxj * maxk, n2 = (size_t)maxi * maxj;
    L.vars.push_back({"longitude", NC_FLOAT, {1}, {{"units", "degrees_east"}, {"long_name", "longitude"}}, (size_t)maxi});
    L.vars.push_back({"latitude", NC_FLOAT, {2}, {{"units", "degrees_north"}, {"long_name", "latitude"}}, (size_t)maxj});
    L.vars.push_back({"depth", NC_FLOAT, {3}, {}, (size_t)maxk});
    for (const char *s : {"ioffset", "iyear", "imonth", "iday"}) L.vars.push_back({s, NC_INT, {0}, {}, 1});
    if (gui) L.vars.push_back({"istep_ocn", NC_INT, {0}, {}, 1});
    for (const char *s : {"temp", "salinity", "uvel", "vvel"}) L.vars.push_back({s, NC_DOUBLE, {3, 2, 1}, {}, n3});
    for (const char *s : {"evap", "late", "sens"}) L.vars.push_back({s, NC_DOUBLE, {2, 1}, {}, n2});
    L.place();
    return L;
}

int nint(double x) { return (int)std::lround(x); }   // Fortran NINT: halves away from zero

uint64_t dbits(double x)
{
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}

// Host part of a restart image: header, coordinates, calendar scalars and the 2-D fluxes.
// The four 3-D fields are filled by the caller (from the host or from the device).
int fill_image(uint8_t *img, const NcLayout &L, int maxi, int maxj, int maxk, const gb_rs_calendar *cal, int gui,
               const double *lon, const double *lat, const double *depths1, const double *evap, const double *late,
               const double *sens)
{
    // every byte after the header belongs to a variable and is written below (all types are
    // 4 or 8 bytes wide, so no variable has padding)
    const std::vector<uint8_t> h = L.header();
    std::memcpy(img, h.data(), h.size());
    const double *axes[3] = {lon, lat, depths1};
    const char *axis_names[3] = {"longitude", "latitude", "depth"};
    const int axis_n[3] = {maxi, maxj, maxk};
    for (int a = 0; a < 3; ++a) {
        uint8_t *p = img + L.var(axis_names[a]).begin;
        for (int i = 0; i < axis_n[a]; ++i) {
            const double x = axes[a][i];
            if (std::isfinite(x) && std::fabs(x) > 3.4028234663852886e38)
                return rs_fail(GB_GO_EINVAL, std::string(axis_names[a]) + " value out of the float range");
            const float f = (float)x;
            uint32_t u;
            std::memcpy(&u, &f, 4);
            store_be(p + 4 * (size_t)i, u, 4);
        }
    }
    const int32_t scal[5] = {cal->ioffset, cal->iyear, cal->imonth, nint(cal->day), cal->istep};
    const char *scal_names[5] = {"ioffset", "iyear", "imonth", "iday", "istep_ocn"};
    for (int s = 0; s < (gui ? 5 : 4); ++s) store_be(img + L.var(scal_names[s]).begin, (uint32_t)scal[s], 4);
    const double *flux[3] = {evap, late, sens};
    const char *flux_names[3] = {"evap", "late", "sens"};
    const size_t n2 = (size_t)maxi * maxj;
    for (int f = 0; f < 3; ++f) {
        uint8_t *p = img + L.var(flux_names[f]).begin;
        for (size_t c = 0; c < n2; ++c) store_be(p + 8 * c, flux[f] ? dbits(flux[f][c]) : 0, 8);
    }
    return GB_GO_OK;
}

int write_file(const char *path, const uint8_t *img, size_t n)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return rs_fail(GB_GO_EINVAL, std::string("cannot create ") + path);
    const size_t w = std::fwrite(img, 1, n, f);
    const int c = std::fclose(f);
    if (w != n || c != 0) return rs_fail(GB_GO_EINVAL, std::string("write failed: ") + path);
    return GB_GO_OK;
}

// The classic format gives a variable's size in 32 bits; only the last fixed-size variable
// may exceed 4 GiB - 4 bytes (its size field then reads 0xFFFFFFFF).  temp, salinity, uvel and
// vvel (8 bytes per cell) are followed by the surface fluxes, so like the netCDF library
// (NC_EVARSIZE) grids of more than 536,870,911 cells are refused.
int check_dims(int maxi, int maxj, int maxk)
{
    if (maxi < 1 || maxj < 1 || maxk < 1)
        return rs_fail(GB_GO_EINVAL, "grid size out of range");
    if ((long long)maxi * maxj * maxk > 536870911LL)
        return rs_fail(GB_GO_EINVAL, "grid too large for the netCDF classic format: a 3-D variable other than the "
                                     "last would exceed 4 GiB - 4 bytes");
    return GB_GO_OK;
}

// ---------------------------------------------------------------- device: the 3-D fields
__device__ __forceinline__ unsigned long long bswap64(unsigned long long v)
{
    const unsigned lo = __byte_perm((unsigned)v, 0u, 0x0123);
    const unsigned hi = __byte_perm((unsigned)(v >> 32), 0u, 0x0123);
    return ((unsigned long long)lo << 32) | hi;
}

// temp, salinity, uvel, vvel of outm_netcdf (goldstein_data.f90:200-213) of one cell c.
struct PackedCell {
    double t, s, u, v;
};

__device__ __forceinline__ PackedCell pack_load(size_t c, const double *__restrict__ ts_static,
                                                const double *__restrict__ cur, int use_cur,
                                                const double *__restrict__ u, const int32_t *__restrict__ k1,
                                                const Dims &d)
{
    const int i = (int)(c % d.maxi) + 1;
    const int j = (int)((c / d.maxi) % d.maxj) + 1;
    const int k = (int)(c / ((size_t)d.maxi * d.maxj)) + 1;
    const int kk = k1[i + d.NI * j];
    const double landmask = kk <= d.maxk ? 1.0 : 0.0;   // the whole column of a wet column
    const double *src = (use_cur && k >= kk) ? cur : ts_static;
    const size_t t = ts_index(d, 0, i, j, k);
    const size_t q = u_index(d, 0, i, j, k);
    return PackedCell{src[t] * landmask, src[t + 1] * landmask, u[q], u[q + 1]};
}

__device__ __forceinline__ void pack_store(unsigned long long *__restrict__ out, size_t n, size_t c, const PackedCell &p)
{
    out[c] = bswap64((unsigned long long)__double_as_longlong(p.t));
    out[n + c] = bswap64((unsigned long long)__double_as_longlong(p.s));
    out[2 * n + c] = bswap64((unsigned long long)__double_as_longlong(p.u));
    out[3 * n + c] = bswap64((unsigned long long)__double_as_longlong(p.v));
}

// One thread per pair of cells a grid-stride apart (both cells' loads are issued before the
// stores), written big-endian one field after another: the data sections of the four variables.
__global__ void k_rs_pack(unsigned long long *__restrict__ out, const double *__restrict__ ts_static,
                          const double *__restrict__ cur, int use_cur, const double *__restrict__ u,
                          const int32_t *__restrict__ k1, Dims d)
{
    const size_t n = (size_t)d.maxi * d.maxj * d.maxk;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c0 < n; c0 += 2 * stride) {
        const size_t c1 = c0 + stride;
        const PackedCell p0 = pack_load(c0, ts_static, cur, use_cur, u, k1, d);
        if (c1 < n) {
            const PackedCell p1 = pack_load(c1, ts_static, cur, use_cur, u, k1, d);
            pack_store(out, n, c0, p0);
            pack_store(out, n, c1, p1);
        } else {
            pack_store(out, n, c0, p0);
        }
    }
}

// ---------------------------------------------------------------- reader
struct NcFile {
    std::vector<uint8_t> bytes;
    int version = 0;
    uint64_t numrecs = 0;
    std::vector<std::pair<std::string, uint64_t>> dims;
    struct Var {
        std::string name;
        std::vector<uint32_t> dimids;
        int type;
        uint64_t begin;
    };
    std::vector<Var> vars;
    size_t pos = 0;
    std::string err;

    bool need(size_t n)
    {
        if (pos + n > bytes.size()) {
            err = "truncated header";
            return false;
        }
        return true;
    }
    bool u32(uint64_t &v)
    {
        if (!need(4)) return false;
        v = load_be(&bytes[pos], 4);
        pos += 4;
        return true;
    }
    bool name(std::string &s)
    {
        uint64_t n;
        if (!u32(n) || !need(pad4(n))) return false;
        s.assign((const char *)&bytes[pos], (size_t)n);
        pos += pad4(n);
        return true;
    }
    bool skip_atts()
    {
        uint64_t tag, n;
        if (!u32(tag) || !u32(n)) return false;
        if (tag != kTagAtt && !(tag == 0 && n == 0)) {
            err = "bad attribute list";
            return false;
        }
        for (uint64_t a = 0; a < n; ++a) {
            std::string nm;
            uint64_t t, ne;
            if (!name(nm) || !u32(t) || !u32(ne)) return false;
            const int ts = type_size((int)t);
            if (!ts) {
                err = "bad attribute type";
                return false;
            }
            if (ne > bytes.size() || !need(pad4(ne * ts))) return false;
            pos += pad4(ne * ts);
        }
        return true;
    }
    bool parse()
    {
        if (bytes.size() >= 4 && bytes[0] == 0x89 && bytes[1] == 'H' && bytes[2] == 'D' && bytes[3] == 'F') {
            err = "netCDF-4 (HDF5) file: needs the netCDF library";
            return false;
        }
        if (bytes.size() < 8 || bytes[0] != 'C' || bytes[1] != 'D' || bytes[2] != 'F') {
            err = "not a netCDF classic file";
            return false;
        }
        version = bytes[3];
        if (version != 1 && version != 2) {
            err = "netCDF format version " + std::to_string(version) + " not supported (CDF-1 and CDF-2 are)";
            return false;
        }
        pos = 4;
        uint64_t tag, n;
        if (!u32(numrecs) || !u32(tag) || !u32(n)) return false;
        if (tag != kTagDim && !(tag == 0 && n == 0)) {
            err = "bad dimension list";
            return false;
        }
        for (uint64_t d = 0; d < n; ++d) {
            std::string nm;
            uint64_t len;
            if (!name(nm) || !u32(len)) return false;
            dims.push_back({nm, len});
        }
        if (!skip_atts()) return false;
        if (!u32(tag) || !u32(n)) return false;
        if (tag != kTagVar && !(tag == 0 && n == 0)) {
            err = "bad variable list";
            return false;
        }
        for (uint64_t v = 0; v < n; ++v) {
            Var var;
            uint64_t nd, t, vs, b;
            if (!name(var.name) || !u32(nd)) return false;
            if (nd > 64) {
                err = "too many dimensions";
                return false;
            }
            for (uint64_t k = 0; k < nd; ++k) {
                uint64_t id;
                if (!u32(id)) return false;
                if (id >= dims.size()) {
                    err = "bad dimension id";
                    return false;
                }
                var.dimids.push_back((uint32_t)id);
            }
            if (!skip_atts() || !u32(t) || !u32(vs)) return false;
            if (version == 1) {
                if (!u32(b)) return false;
            } else {
                if (!need(8)) return false;
                b = load_be(&bytes[pos], 8);
                pos += 8;
            }
            var.type = (int)t;
            var.begin = b;
            vars.push_back(var);
        }
        return true;
    }
    const Var *find(const char *nm) const
    {
        for (const auto &v : vars)
            if (v.name == nm) return &v;
        return nullptr;
    }
    // the values of `nm` as doubles; shape (slowest first) must be `want` (the record dimension,
    // length 0 in the list, counts as one record)
    int get(const char *nm, const std::vector<uint64_t> &want, double *out)
    {
        const Var *v = find(nm);
        if (!v) return rs_fail(GB_GO_EINVAL, std::string("variable ") + nm + " missing");
        std::vector<uint64_t> shape;
        for (uint32_t id : v->dimids) shape.push_back(dims[id].second == 0 ? 1 : dims[id].second);
        if (shape != want) return rs_fail(GB_GO_EINVAL, std::string("variable ") + nm + " has another shape");
        const int ts = type_size(v->type);
        if (!ts || v->type == NC_CHAR) return rs_fail(GB_GO_EINVAL, std::string("variable ") + nm + " is not numeric");
        uint64_t n = 1;
        for (uint64_t s : shape) n *= s;
        if (v->begin > bytes.size() || n * ts > bytes.size() - v->begin)
            return rs_fail(GB_GO_EINVAL, std::string("variable ") + nm + " beyond the end of the file");
        const uint8_t *p = &bytes[v->begin];
        for (uint64_t e = 0; e < n; ++e) {
            const uint64_t raw = load_be(p + e * ts, ts);
            double x;
            switch (v->type) {
            case NC_BYTE: x = (double)(int8_t)(uint8_t)raw; break;
            case NC_SHORT: x = (double)(int16_t)(uint16_t)raw; break;
            case NC_INT: x = (double)(int32_t)(uint32_t)raw; break;
            case NC_FLOAT: {
                const uint32_t r32 = (uint32_t)raw;
                float f;
                std::memcpy(&f, &r32, 4);
                x = (double)f;
                break;
            }
            default: std::memcpy(&x, &raw, 8); break;
            }
            out[e] = x;
        }
        return GB_GO_OK;
    }
    int get_int(const char *nm, int32_t *out)
    {
        double x;
        const int r = get(nm, {1}, &x);
        if (r) return r;
        if (!(x >= -2147483648.0 && x < 2147483648.0)) return rs_fail(GB_GO_EINVAL, std::string(nm) + " out of the int range");
        *out = (int32_t)x;   // conversion to int truncates, as the netCDF library's does
        return GB_GO_OK;
    }
};

void advance(gb_rs_calendar *cal, int iday, double step_days)
{
    cal->day = cal->day + step_days;
    if (std::fabs((double)iday - cal->day) <= 1.0e-3) cal->day = (double)iday;
    if (cal->day >= 31.0) {
        cal->day = cal->day - 30.0;
        cal->imonth = cal->imonth + 1;
        if (cal->imonth == 13) {
            cal->imonth = 1;
            cal->iyear = cal->iyear + 1;
        }
    }
}

// Staging buffers of the writer, kept between calls (a restart of a large grid would otherwise
// pin and free tens of MB each time): one pinned file image and one device buffer per device.
std::mutex g_stage_mutex;
struct Stage {
    uint8_t *host = nullptr;
    size_t host_bytes = 0;
    void *dev = nullptr;
    size_t dev_bytes = 0;
};
std::map<int, Stage> g_stage;

cudaError_t stage_buffers(int device, size_t host_bytes, size_t dev_bytes, uint8_t **host, void **dev)
{
    Stage &st = g_stage[device];
    if (st.host_bytes < host_bytes) {
        if (st.host) cudaFreeHost(st.host);
        st.host = nullptr;
        st.host_bytes = 0;
        cudaError_t e = cudaMallocHost((void **)&st.host, host_bytes);
        if (e != cudaSuccess) return e;
        st.host_bytes = host_bytes;
    }
    if (st.dev_bytes < dev_bytes) {
        if (st.dev) cudaFree(st.dev);
        st.dev = nullptr;
        st.dev_bytes = 0;
        cudaError_t e = cudaMalloc(&st.dev, dev_bytes);
        if (e != cudaSuccess) return e;
        st.dev_bytes = dev_bytes;
    }
    *host = st.host;
    *dev = st.dev;
    return cudaSuccess;
}

}  // namespace

#define RS_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            rc = rs_fail(GB_GO_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
            goto done;                                                                     \
        }                                                                                  \
    } while (0)

extern "C" const char *gb_rs_last_error(void) { return g_err.c_str(); }

extern "C" int gb_rs_write_fields(const char *path, int32_t maxi, int32_t maxj, int32_t maxk, const gb_rs_calendar *cal,
                                  int32_t gui, const double *lon, const double *lat, const double *depths1,
                                  const double *temp, const double *salinity, const double *uvel, const double *vvel,
                                  const double *evap, const double *late, const double *sens)
{
    gbgo::TraceRange tr_("rs_write_fields");
    if (!path || !cal || !lon || !lat || !depths1 || !temp || !salinity || !uvel || !vvel)
        return rs_fail(GB_GO_EINVAL, "write_fields: NULL argument");
    if (int r = check_dims(maxi, maxj, maxk)) return r;
    const NcLayout L = goldstein_layout(maxi, maxj, maxk, gui);
    std::vector<uint8_t> img(L.total_bytes);
    if (int r = fill_image(img.data(), L, maxi, maxj, maxk, cal, gui, lon, lat, depths1, evap, late, sens)) return r;
    const double *f3[4] = {temp, salinity, uvel, vvel};
    const char *n3[4] = {"temp", "salinity", "uvel", "vvel"};
    const size_t n = (size_t)maxi * maxj * maxk;
    for (int f = 0; f < 4; ++f) {
        uint8_t *p = img.data() + L.var(n3[f]).begin;
        for (size_t c = 0; c < n; ++c) store_be(p + 8 * c, dbits(f3[f][c]), 8);
    }
    return write_file(path, img.data(), img.size());
}

namespace {
// Validates the ocean handle and enqueues k_rs_pack on its stream (after the split-precision
// form's export), writing the four 3-D variables to `dev` (4 * maxi*maxj*maxk words).
int pack_fields(gb_go_handle *ocean, unsigned long long *dev, OceanState &o, bool export_state = true)
{
    if (ocean_state(ocean, &o) != GB_GO_OK) return rs_fail(GB_GO_EINVAL, "restart: bad ocean handle");
    if (!o.state_ready) return rs_fail(GB_GO_ENOTREADY, "restart: ocean state not uploaded");
    if (o.d.L < 2) return rs_fail(GB_GO_EINVAL, "restart: the ocean has no T and S");
    if (int r = check_dims(o.d.maxi, o.d.maxj, o.d.maxk)) return r;
    cudaError_t e = cudaSetDevice(o.device);
    if (e != cudaSuccess) return rs_fail(GB_GO_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    if (const int rr = export_state ? ocean_refresh_rho(ocean) : GB_GO_OK)   // the split-precision form exports its state
        return rs_fail(rr, std::string("restart: state export failed: ") + gb_go_last_error(ocean));
    if (!dev) return GB_GO_OK;
    const size_t n = (size_t)o.d.maxi * o.d.maxj * o.d.maxk;
    // two cells per thread; at most one wave of 8 resident 256-thread blocks on each of 152 SMs
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 511) / 512, 152 * 8));
    k_rs_pack<<<blocks, 256, 0, (cudaStream_t)o.stream>>>(dev, o.ts_static, o.ts_buf[o.cur], o.steps_since_upload > 0 ? 1 : 0,
                                                         o.u, o.k1, o.d);
    count_launches(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return rs_fail(GB_GO_ECUDA, std::string("k_rs_pack: ") + cudaGetErrorString(e));
    return GB_GO_OK;
}
}  // namespace

extern "C" int gb_rs_pack_goldstein(gb_go_handle *ocean, void *dev_out)
{
    if (!ocean || !dev_out) return rs_fail(GB_GO_EINVAL, "pack_goldstein: NULL argument");
    if (((uintptr_t)dev_out) % 8) return rs_fail(GB_GO_EINVAL, "pack_goldstein: dev_out not 8-byte aligned");
    OceanState o;
    return pack_fields(ocean, (unsigned long long *)dev_out, o);
}

extern "C" int gb_rs_write_goldstein(gb_go_handle *ocean, const char *path, const gb_rs_calendar *cal, int32_t gui,
                                     const double *nclon1, const double *nclat1, const double *ncdepth,
                                     const double *evap, const double *late, const double *sens)
{
    gbgo::TraceRange tr_("rs_write_goldstein");
    if (!ocean || !path || !cal || !nclon1 || !nclat1 || !ncdepth) return rs_fail(GB_GO_EINVAL, "write_goldstein: NULL argument");
    OceanState o;
    if (int r = pack_fields(ocean, nullptr, o)) return r;   // validation and export only
    const int maxi = o.d.maxi, maxj = o.d.maxj, maxk = o.d.maxk;
    const NcLayout L = goldstein_layout(maxi, maxj, maxk, gui);
    const size_t n = (size_t)maxi * maxj * maxk;
    std::vector<double> depths1(maxk);
    for (int k = 0; k < maxk; ++k) depths1[k] = ncdepth[maxk - 1 - k];
    uint8_t *img = nullptr;
    unsigned long long *dev = nullptr;
    int rc = GB_GO_OK;
    cudaStream_t s = (cudaStream_t)o.stream;
    std::lock_guard<std::mutex> lock(g_stage_mutex);   // the staging buffers are shared
    RS_CUDA(stage_buffers(o.device, L.total_bytes, 4 * n * sizeof(unsigned long long), &img, (void **)&dev));
    rc = pack_fields(ocean, dev, o, false);   // exported above
    if (rc) goto done;
    rc = fill_image(img, L, maxi, maxj, maxk, cal, gui, nclon1, nclat1, depths1.data(), evap, late, sens);
    if (rc) goto done;
    // the four 3-D variables are consecutive in the file: one copy
    RS_CUDA(cudaMemcpyAsync(img + L.var("temp").begin, dev, 4 * n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    RS_CUDA(cudaStreamSynchronize(s));
    rc = write_file(path, img, L.total_bytes);
done:
    return rc;
}

extern "C" int gb_rs_read_goldstein(const char *path, int32_t maxi, int32_t maxj, int32_t maxk, int32_t gui,
                                    gb_rs_calendar *cal, double *temp, double *salinity, double *uvel, double *vvel,
                                    double *evap, double *late, double *sens)
{
    gbgo::TraceRange tr_("rs_read_goldstein");
    if (!path) return rs_fail(GB_GO_EINVAL, "read_goldstein: NULL path");
    if (int r = check_dims(maxi, maxj, maxk)) return r;
    NcFile f;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return rs_fail(GB_GO_EINVAL, std::string("missing file ") + path);
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    if (sz > 0) {
        f.bytes.resize((size_t)sz);
        if (std::fread(f.bytes.data(), 1, (size_t)sz, fp) != (size_t)sz) {
            std::fclose(fp);
            return rs_fail(GB_GO_EINVAL, std::string("read failed: ") + path);
        }
    }
    std::fclose(fp);
    if (!f.parse()) {
        const bool unsupported = f.err.find("HDF5") != std::string::npos || f.err.find("version") != std::string::npos;
        return rs_fail(unsupported ? GB_GO_EUNSUPPORTED : GB_GO_EINVAL, std::string(path) + ": " + f.err);
    }
    if (cal) {
        int32_t iday = 0;
        if (gui) {
            if (int r = f.get_int("istep_ocn", &cal->istep)) return r;
        }
        if (int r = f.get_int("ioffset", &cal->ioffset)) return r;
        if (int r = f.get_int("iyear", &cal->iyear)) return r;
        if (int r = f.get_int("imonth", &cal->imonth)) return r;
        if (int r = f.get_int("iday", &iday)) return r;
        cal->day = (double)iday;
    }
    const std::vector<uint64_t> s3 = {(uint64_t)maxk, (uint64_t)maxj, (uint64_t)maxi}, s2 = {(uint64_t)maxj, (uint64_t)maxi};
    double *o3[4] = {temp, salinity, uvel, vvel};
    const char *n3[4] = {"temp", "salinity", "uvel", "vvel"};
    for (int v = 0; v < 4; ++v)
        if (o3[v])
            if (int r = f.get(n3[v], s3, o3[v])) return r;
    double *o2[3] = {evap, late, sens};
    const char *n2[3] = {"evap", "late", "sens"};
    for (int v = 0; v < 3; ++v)
        if (o2[v])
            if (int r = f.get(n2[v], s2, o2[v])) return r;
    return GB_GO_OK;
}

extern "C" int gb_rs_goldstein_name(const char *dir, const gb_rs_calendar *cal, char *out, int32_t out_len)
{
    if (!dir || !cal || !out || out_len <= 0) return rs_fail(GB_GO_EINVAL, "goldstein_name: NULL argument");
    // Fortran edit descriptors: i10 for the year (left-adjusted, trimmed), i2.2 for month and day
    char year[16], month[4], day[4];
    std::snprintf(year, sizeof(year), "%d", cal->iyear);
    if (std::strlen(year) > 10) std::snprintf(year, sizeof(year), "**********");
    const int iday = nint(cal->day);
    if (cal->imonth >= 0 && cal->imonth <= 99) std::snprintf(month, sizeof(month), "%02d", cal->imonth);
    else std::snprintf(month, sizeof(month), "**");
    if (iday >= 0 && iday <= 99) std::snprintf(day, sizeof(day), "%02d", iday);
    else std::snprintf(day, sizeof(day), "**");
    const std::string name = std::string(dir) + "/goldstein_restart_" + year + "_" + month + "_" + day + ".nc";
    if ((int64_t)name.size() + 1 > out_len) return rs_fail(GB_GO_EINVAL, "goldstein_name: buffer too small");
    std::memcpy(out, name.c_str(), name.size() + 1);
    return (int)name.size();
}

extern "C" void gb_rs_calendar_step(gb_rs_calendar *cal, double yearlen, int32_t nyear)
{
    if (!cal) return;
    const double timestep = yearlen / (double)nyear;
    const int iday = nint(cal->day);
    advance(cal, iday, timestep);
}

extern "C" void gb_rs_calendar_after_read(gb_rs_calendar *cal, double yearlen, int32_t nyear)
{
    if (!cal) return;
    const double timestep = 24.0 * 60.0 * 60.0 * yearlen / (double)nyear;
    const int iday = (int)cal->day;
    cal->day = (double)iday;
    const int ylen = nint(yearlen);
    if (ylen != 0) cal->ioffset = cal->ioffset % ylen;
    advance(cal, iday, timestep / (24 * 60 * 60.0));
}
