// k_output.cu -- VTK XML RectilinearGrid output of device-resident fields
// (include/scf_output.h), the file PrintResultVTK writes
// (src/PrintResult.f90:328-421): node coordinates in Float32, cell data
// rounded to Float32 in i-fastest order.  A kernel gathers each field's
// interior cells and rounds them on the device, so half the bytes cross to
// the host; fields are pipelined through two device and two page-locked
// buffers, so the conversion and copy of one field overlap the file write of
// the previous one.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/scf_output.h"
#include "scf_common.cuh"
#include "scf_devmem.h"

namespace {

// One block row of 256 cells along i of one (j, k) line per block:
// grid (ceil(I/256), J, K), no index division.
__global__ void __launch_bounds__(256) k_gather_f32(const double *__restrict__ src, float *__restrict__ dst, int I,
                                                    int J)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= I) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const long long g = (i + 1) + (long long)(I + 2) * ((j + 1) + (long long)(J + 2) * (k + 1));
    dst[i + (long long)I * (j + (long long)J * k)] = __double2float_rn(src[g]);
}

// Base64 (RFC 4648, '=' padding), the encoding of VTKFortran's "BINARY"
// data arrays (BeFoR64's b64_encode): of the byte stream H || data, where H
// is the Int32 byte count of the data (little endian) that VTKFortran packs
// in front (encode_binary_dataarray).  Thread g forms the 4 characters of
// bytes 3g .. 3g+2 of the stream.
__constant__ char c_b64[65] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

__device__ __forceinline__ unsigned stream_byte(const unsigned char *data, unsigned hdr, long long B, long long pos)
{
    if (pos < 4) return (hdr >> (8 * pos)) & 0xffu;
    return pos < B ? data[pos - 4] : 0u;
}

__global__ void __launch_bounds__(256) k_b64(const unsigned char *__restrict__ data, unsigned hdr, long long B,
                                             long long G, char *__restrict__ out)
{
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += (long long)gridDim.x * blockDim.x) {
        const long long p0 = 3 * g;
        const unsigned b0 = stream_byte(data, hdr, B, p0), b1 = stream_byte(data, hdr, B, p0 + 1),
                       b2 = stream_byte(data, hdr, B, p0 + 2);
        char4 c;
        c.x = c_b64[b0 >> 2];
        c.y = c_b64[((b0 & 3u) << 4) | (b1 >> 4)];
        c.z = p0 + 1 < B ? c_b64[((b1 & 15u) << 2) | (b2 >> 6)] : '=';
        c.w = p0 + 2 < B ? c_b64[b2 & 63u] : '=';
        reinterpret_cast<char4 *>(out)[g] = c;
    }
}

// The same encoding on the host (the small coordinate arrays).
std::string b64_host(const void *data, size_t nbytes)
{
    static const char A[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::vector<unsigned char> s(4 + nbytes);
    const unsigned hdr = (unsigned)nbytes;
    for (int q = 0; q < 4; ++q) s[q] = (unsigned char)((hdr >> (8 * q)) & 0xffu);
    std::memcpy(s.data() + 4, data, nbytes);
    std::string out;
    out.reserve((s.size() + 2) / 3 * 4);
    for (size_t p = 0; p < s.size(); p += 3) {
        const unsigned b0 = s[p], b1 = p + 1 < s.size() ? s[p + 1] : 0u, b2 = p + 2 < s.size() ? s[p + 2] : 0u;
        out += A[b0 >> 2];
        out += A[((b0 & 3u) << 4) | (b1 >> 4)];
        out += p + 1 < s.size() ? A[((b1 & 15u) << 2) | (b2 >> 6)] : '=';
        out += p + 2 < s.size() ? A[b2 & 63u] : '=';
    }
    return out;
}

bool name_ok(const char *s)
{
    if (!s || !*s) return false;
    for (; *s; ++s)
        if (*s == '"' || *s == '<' || *s == '&' || *s == '>') return false;
    return true;
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Node coordinates of one axis as PrintResultVTK forms them (Float32 of the
// FP64 expressions).
std::vector<float> nodes(const double *c, const double *w, int n)
{
    std::vector<float> x(n + 1);
    for (int i = 0; i < n; ++i) x[i] = (float)(c[i] - w[i] / 2.0);
    x[n] = (float)(c[n - 1] + w[n - 1] / 2.0);
    return x;
}

struct Cleanup {
    std::vector<void *> dev, host;
    std::vector<cudaStream_t> st;
    std::vector<cudaEvent_t> ev;
    FILE *f = nullptr;
    ~Cleanup()
    {
        for (auto s : st) cudaStreamSynchronize(s);
        for (void *p : dev) scf_mem::dev_free(p);
        for (void *p : host) cudaFreeHost(p);
        for (auto e : ev) cudaEventDestroy(e);
        for (auto s : st) cudaStreamDestroy(s);
        if (f) fclose(f);
    }
};

}  // namespace

namespace {

// The two layouts: raw Float32 arrays in an appended section with UInt64
// byte counts, or VTKFortran's "BINARY" layout (each array inline, base64
// of its Int32 byte count and the data), which is what PrintResultVTK's
// initialize(format='BINARY') writes.
enum VtrMode { VTR_APPENDED = 0, VTR_BINARY = 1 };

// VTKFortran's text for the inline mode: tags indented by 2 per level, a
// data array's base64 on its own line indented 2 deeper, integers in the
// extents with PENF's explicit '+' sign (str(n=...)).
std::string binary_array_head(const char *name)
{
    return std::string("        <DataArray type=\"Float32\" NumberOfComponents=\"1\" Name=\"") + name +
           "\" format=\"binary\">\n          ";
}
const char *const kBinaryArrayTail = "\n        </DataArray>\n";

// The inline (base64) file.  Fields go through two slots, each a device
// Float32 buffer, a device character buffer and a page-locked host
// character buffer, on two streams: gather + round, encode, copy out; the
// host writes field q-1 while field q is prepared.
int write_binary(const char *path, int imax, int jmax, int kmax, const std::vector<float> &X,
                 const std::vector<float> &Y, const std::vector<float> &Z, long long n, long long ng, int nfields,
                 const scf_vtr_field *fields, scf_vtr_stats *stats, std::chrono::steady_clock::time_point t0)
{
    char buf[256];
    std::snprintf(buf, sizeof buf, "+%d +%d +%d +%d +%d +%d", 1, imax + 1, 1, jmax + 1, 1, kmax + 1);
    const std::string ext(buf);
    std::string h;
    h += "<?xml version=\"1.0\"?>\n";
    h += "<VTKFile type=\"RectilinearGrid\" version=\"1.0\" byte_order=\"LittleEndian\">\n";
    h += "  <RectilinearGrid WholeExtent=\"" + ext + "\">\n";
    h += "    <Piece Extent=\"" + ext + "\">\n";
    h += "      <Coordinates>\n";
    h += binary_array_head("X") + b64_host(X.data(), 4 * X.size()) + kBinaryArrayTail;
    h += binary_array_head("Y") + b64_host(Y.data(), 4 * Y.size()) + kBinaryArrayTail;
    h += binary_array_head("Z") + b64_host(Z.data(), 4 * Z.size()) + kBinaryArrayTail;
    h += "      </Coordinates>\n";
    h += "      <CellData>\n";
    const std::string tail = "      </CellData>\n    </Piece>\n  </RectilinearGrid>\n</VTKFile>\n";
    const long long B = 4 + 4 * n;        // bytes of one encoded stream
    const long long G = (B + 2) / 3;      // 3-byte groups, 4 characters each

    Cleanup c;
    c.f = std::fopen(path, "wb");
    if (!c.f) return SCF_ERR_BAD_ARG;
    double ms_write = 0.0, ms_d2h = 0.0;
    float ms_conv = 0.0f;
    int launches = 0;
    long long fbytes = 0;
    auto put = [&](const void *p, size_t bytes) {
        const auto tw = std::chrono::steady_clock::now();
        const bool ok = std::fwrite(p, 1, bytes, c.f) == bytes;
        ms_write += ms_since(tw);
        fbytes += (long long)bytes;
        return ok;
    };
    if (!put(h.data(), h.size())) return SCF_ERR_BAD_ARG;
    if (nfields > 0) {
        float *dbuf[2];
        char *cbuf[2], *hbuf[2];
        double *dsrc[2] = {nullptr, nullptr};
        for (int s = 0; s < 2; ++s) {
            cudaStream_t st;
            cudaEvent_t e0, e1, e2;
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
            c.st.push_back(st);
            if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
                cudaEventCreate(&e2) != cudaSuccess)
                return SCF_ERR_CUDA;
            c.ev.push_back(e0); c.ev.push_back(e1); c.ev.push_back(e2);
            void *p = nullptr;
            if (scf_mem::dev_malloc(&p, sizeof(float) * n) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
            c.dev.push_back(p);
            dbuf[s] = (float *)p;
            if (scf_mem::dev_malloc(&p, (size_t)(4 * G)) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
            c.dev.push_back(p);
            cbuf[s] = (char *)p;
            if (cudaMallocHost(&p, (size_t)(4 * G)) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
            c.host.push_back(p);
            hbuf[s] = (char *)p;
        }
        bool host_fields = false;
        for (int q = 0; q < nfields; ++q) host_fields |= fields[q].on_device == 0;
        if (host_fields)
            for (int s = 0; s < 2; ++s) {
                void *p = nullptr;
                if (scf_mem::dev_malloc(&p, sizeof(double) * ng) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
                c.dev.push_back(p);
                dsrc[s] = (double *)p;
            }
        const dim3 grid((imax + 255) / 256, jmax, kmax);
        const long long want = (G + 255) / 256;
        const int egrid = (int)(want < 152 * 8 ? want : 152 * 8);
        auto issue = [&](int q) {
            const int s = q & 1;
            cudaStream_t st = c.st[s];
            const double *src = fields[q].data;
            if (!fields[q].on_device) {
                cudaMemcpyAsync(dsrc[s], src, sizeof(double) * ng, cudaMemcpyHostToDevice, st);
                src = dsrc[s];
            }
            cudaEventRecord(c.ev[3 * s], st);
            k_gather_f32<<<grid, 256, 0, st>>>(src, dbuf[s], imax, jmax);
            k_b64<<<egrid, 256, 0, st>>>((const unsigned char *)dbuf[s], (unsigned)(4 * n), B, G, cbuf[s]);
            cudaEventRecord(c.ev[3 * s + 1], st);
            cudaMemcpyAsync(hbuf[s], cbuf[s], (size_t)(4 * G), cudaMemcpyDeviceToHost, st);
            cudaEventRecord(c.ev[3 * s + 2], st);
            launches += 2;
        };
        issue(0);
        for (int q = 0; q < nfields; ++q) {
            const int s = q & 1;
            if (q + 1 < nfields) issue(q + 1);
            if (cudaEventSynchronize(c.ev[3 * s + 2]) != cudaSuccess) return SCF_ERR_CUDA;
            float a = 0.f, b = 0.f;
            cudaEventElapsedTime(&a, c.ev[3 * s], c.ev[3 * s + 1]);
            cudaEventElapsedTime(&b, c.ev[3 * s + 1], c.ev[3 * s + 2]);
            ms_conv += a;
            ms_d2h += b;
            const std::string head = binary_array_head(fields[q].name);
            if (!put(head.data(), head.size()) || !put(hbuf[s], (size_t)(4 * G)) ||
                !put(kBinaryArrayTail, std::strlen(kBinaryArrayTail)))
                return SCF_ERR_BAD_ARG;
        }
        if (cudaGetLastError() != cudaSuccess) return SCF_ERR_CUDA;
    }
    if (!put(tail.data(), tail.size())) return SCF_ERR_BAD_ARG;
    {
        const auto tw = std::chrono::steady_clock::now();
        const int rc = std::fclose(c.f);
        c.f = nullptr;
        ms_write += ms_since(tw);
        if (rc != 0) return SCF_ERR_BAD_ARG;
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->ms_convert = ms_conv;
        stats->ms_d2h = ms_d2h;
        stats->ms_write = ms_write;
        stats->ms_total = ms_since(t0);
        stats->bytes_file = fbytes;
        stats->gpu_launches = launches;
    }
    return SCF_OK;
}

int write_vtr_impl(VtrMode mode, const char *path, int32_t imax, int32_t jmax, int32_t kmax, const double *xc,
                   const double *dx, const double *yc, const double *dy, const double *zc, const double *dz,
                   int32_t nfields, const scf_vtr_field *fields, int32_t device, scf_vtr_stats *stats)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (!path || imax < 1 || jmax < 1 || kmax < 1 || jmax > 65535 || kmax > 65535 || !xc || !dx || !yc || !dy || !zc || !dz || nfields < 0 ||
        (nfields > 0 && !fields))
        return SCF_ERR_BAD_ARG;
    for (int q = 0; q < nfields; ++q)
        if (!fields[q].data || !name_ok(fields[q].name)) return SCF_ERR_BAD_ARG;
    const long long n = (long long)imax * jmax * kmax;
    const long long ng = (long long)(imax + 2) * (jmax + 2) * (kmax + 2);
    // the inline layout's byte count is an Int32 (VTKFortran's I4P)
    if (mode == VTR_BINARY && 4 * n > 2147483647LL) return SCF_ERR_BAD_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_NO_DEVICE;
    const std::vector<float> X = nodes(xc, dx, imax), Y = nodes(yc, dy, jmax), Z = nodes(zc, dz, kmax);
    if (mode == VTR_BINARY) return write_binary(path, imax, jmax, kmax, X, Y, Z, n, ng, nfields, fields, stats, t0);

    // XML header; array q's offset counts the UInt64 byte counts before it
    std::string h;
    char buf[512];
    std::snprintf(buf, sizeof buf, "%d %d %d %d %d %d", 1, imax + 1, 1, jmax + 1, 1, kmax + 1);
    const std::string ext(buf);
    h += "<?xml version=\"1.0\"?>\n";
    h += "<VTKFile type=\"RectilinearGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
    h += "  <RectilinearGrid WholeExtent=\"" + ext + "\">\n";
    h += "    <Piece Extent=\"" + ext + "\">\n";
    unsigned long long off = 0;
    auto array = [&](const char *name, unsigned long long bytes) {
        std::snprintf(buf, sizeof buf,
                      "        <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"1\" format=\"appended\" "
                      "offset=\"%llu\"/>\n",
                      name, off);
        off += 8 + bytes;
        return std::string(buf);
    };
    h += "      <Coordinates>\n";
    h += array("X_COORDINATES", 4ull * (imax + 1));
    h += array("Y_COORDINATES", 4ull * (jmax + 1));
    h += array("Z_COORDINATES", 4ull * (kmax + 1));
    h += "      </Coordinates>\n";
    h += "      <CellData>\n";
    for (int q = 0; q < nfields; ++q) h += array(fields[q].name, 4ull * n);
    h += "      </CellData>\n";
    h += "    </Piece>\n";
    h += "  </RectilinearGrid>\n";
    h += "  <AppendedData encoding=\"raw\">\n_";
    const std::string tail = "\n  </AppendedData>\n</VTKFile>\n";

    Cleanup c;
    c.f = std::fopen(path, "wb");
    if (!c.f) return SCF_ERR_BAD_ARG;
    double ms_write = 0.0, ms_d2h = 0.0;
    float ms_conv = 0.0f;
    int launches = 0;
    auto put = [&](const void *p, size_t bytes) {
        const auto tw = std::chrono::steady_clock::now();
        const bool ok = std::fwrite(p, 1, bytes, c.f) == bytes;
        ms_write += ms_since(tw);
        return ok;
    };
    auto put_array = [&](const void *p, unsigned long long bytes) {
        return put(&bytes, 8) && put(p, bytes);
    };
    if (!put(h.data(), h.size()) || !put_array(X.data(), 4ull * X.size()) || !put_array(Y.data(), 4ull * Y.size()) ||
        !put_array(Z.data(), 4ull * Z.size()))
        return SCF_ERR_BAD_ARG;
    if (nfields > 0) {
        float *dbuf[2], *hbuf[2];
        double *dsrc[2] = {nullptr, nullptr};
        for (int s = 0; s < 2; ++s) {
            cudaStream_t st;
            cudaEvent_t e0, e1, e2;
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return SCF_ERR_CUDA;
            c.st.push_back(st);
            if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
                cudaEventCreate(&e2) != cudaSuccess)
                return SCF_ERR_CUDA;
            c.ev.push_back(e0); c.ev.push_back(e1); c.ev.push_back(e2);
            void *p = nullptr;
            if (scf_mem::dev_malloc(&p, sizeof(float) * n) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
            c.dev.push_back(p);
            dbuf[s] = (float *)p;
            if (cudaMallocHost(&p, sizeof(float) * n) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
            c.host.push_back(p);
            hbuf[s] = (float *)p;
        }
        bool host_fields = false;
        for (int q = 0; q < nfields; ++q) host_fields |= fields[q].on_device == 0;
        if (host_fields)
            for (int s = 0; s < 2; ++s) {
                void *p = nullptr;
                if (scf_mem::dev_malloc(&p, sizeof(double) * ng) != cudaSuccess) return SCF_ERR_OUT_OF_MEMORY;
                c.dev.push_back(p);
                dsrc[s] = (double *)p;
            }
        const dim3 grid((imax + 255) / 256, jmax, kmax);
        // field q on slot q%2: [host copy in] gather+round, D2H; the host
        // writes field q-1 while field q converts and copies
        auto issue = [&](int q) {
            const int s = q & 1;
            cudaStream_t st = c.st[s];
            const double *src = fields[q].data;
            if (!fields[q].on_device) {
                cudaMemcpyAsync(dsrc[s], src, sizeof(double) * ng, cudaMemcpyHostToDevice, st);
                src = dsrc[s];
            }
            cudaEventRecord(c.ev[3 * s], st);
            k_gather_f32<<<grid, 256, 0, st>>>(src, dbuf[s], imax, jmax);
            cudaEventRecord(c.ev[3 * s + 1], st);
            cudaMemcpyAsync(hbuf[s], dbuf[s], sizeof(float) * n, cudaMemcpyDeviceToHost, st);
            cudaEventRecord(c.ev[3 * s + 2], st);
            ++launches;
        };
        issue(0);
        for (int q = 0; q < nfields; ++q) {
            const int s = q & 1;
            if (q + 1 < nfields) issue(q + 1);
            if (cudaEventSynchronize(c.ev[3 * s + 2]) != cudaSuccess) return SCF_ERR_CUDA;
            float a = 0.f, b = 0.f;
            cudaEventElapsedTime(&a, c.ev[3 * s], c.ev[3 * s + 1]);
            cudaEventElapsedTime(&b, c.ev[3 * s + 1], c.ev[3 * s + 2]);
            ms_conv += a;
            ms_d2h += b;
            if (!put_array(hbuf[s], 4ull * n)) return SCF_ERR_BAD_ARG;
        }
        if (cudaGetLastError() != cudaSuccess) return SCF_ERR_CUDA;
    }
    if (!put(tail.data(), tail.size())) return SCF_ERR_BAD_ARG;
    const long long fbytes = (long long)h.size() + (long long)tail.size() + 3 * 8 +
                             4ll * (X.size() + Y.size() + Z.size()) + (long long)nfields * (8 + 4 * n);
    {
        const auto tw = std::chrono::steady_clock::now();
        const int rc = std::fclose(c.f);
        c.f = nullptr;
        ms_write += ms_since(tw);
        if (rc != 0) return SCF_ERR_BAD_ARG;
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->ms_convert = ms_conv;
        stats->ms_d2h = ms_d2h;
        stats->ms_write = ms_write;
        stats->ms_total = ms_since(t0);
        stats->bytes_file = fbytes;
        stats->gpu_launches = launches;
    }
    return SCF_OK;
}

}  // namespace

extern "C" int scf_write_vtr(const char *path, int32_t imax, int32_t jmax, int32_t kmax, const double *xc,
                             const double *dx, const double *yc, const double *dy, const double *zc, const double *dz,
                             int32_t nfields, const scf_vtr_field *fields, int32_t device, scf_vtr_stats *stats)
{
    return write_vtr_impl(VTR_APPENDED, path, imax, jmax, kmax, xc, dx, yc, dy, zc, dz, nfields, fields, device,
                          stats);
}

extern "C" int scf_write_vtr_binary(const char *path, int32_t imax, int32_t jmax, int32_t kmax, const double *xc,
                                    const double *dx, const double *yc, const double *dy, const double *zc,
                                    const double *dz, int32_t nfields, const scf_vtr_field *fields, int32_t device,
                                    scf_vtr_stats *stats)
{
    return write_vtr_impl(VTR_BINARY, path, imax, jmax, kmax, xc, dx, yc, dy, zc, dz, nfields, fields, device, stats);
}
