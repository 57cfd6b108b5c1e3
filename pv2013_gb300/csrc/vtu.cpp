// VTK XML unstructured-grid writer for point data (.vtu), the file type the
// reference writes with VTK (OutputFile.cpp:16-137): one VTK_VERTEX cell per
// point, Float32 point coordinates, Float64 point arrays.  Written with raw
// appended binary data (UInt64 block headers, little-endian), which ParaView
// and the VTK readers load directly.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "lbm_gb300.h"

using namespace lbm;

namespace {

struct Out {
    FILE* f;
    bool ok = true;
    void put(const std::string& s) { ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size(); }
    void raw(const void* p, size_t bytes) {
        const uint64_t h = bytes;
        ok = ok && std::fwrite(&h, sizeof h, 1, f) == 1;
        if (bytes) ok = ok && std::fwrite(p, 1, bytes, f) == bytes;
    }
};

}  // namespace

extern "C" lbm_status lbm_vtu_write(const char* path, size_t n, const float* xyz, size_t narrays,
                                    const lbm_vtu_array* arrays) {
    if (!path || (n && !xyz) || (narrays && !arrays)) return fail(LBM_ERR_ARG, "lbm_vtu_write: null argument");
    for (size_t a = 0; a < narrays; ++a)
        if (!arrays[a].name || arrays[a].components < 1 || (n && !arrays[a].data))
            return fail(LBM_ERR_ARG, "lbm_vtu_write: array %zu is incomplete", a);
    clear_error();
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(LBM_ERR_IO, "cannot open %s for writing: %s", path, std::strerror(errno));
    Out o{f};
    // appended block offsets: each block is an 8-byte length plus the data
    uint64_t off = 0;
    std::vector<uint64_t> offs;
    for (size_t a = 0; a < narrays; ++a) {
        offs.push_back(off);
        off += 8 + (uint64_t)n * arrays[a].components * sizeof(double);
    }
    const uint64_t off_pts = off;  off += 8 + (uint64_t)n * 3 * sizeof(float);
    const uint64_t off_con = off;  off += 8 + (uint64_t)n * sizeof(int64_t);
    const uint64_t off_ofs = off;  off += 8 + (uint64_t)n * sizeof(int64_t);
    const uint64_t off_typ = off;
    char buf[512];
    o.put("<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
          "header_type=\"UInt64\">\n  <UnstructuredGrid>\n");
    std::snprintf(buf, sizeof buf, "    <Piece NumberOfPoints=\"%zu\" NumberOfCells=\"%zu\">\n      <PointData>\n", n, n);
    o.put(buf);
    for (size_t a = 0; a < narrays; ++a) {
        std::snprintf(buf, sizeof buf,
                      "        <DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"appended\" "
                      "offset=\"%llu\"/>\n",
                      arrays[a].name, arrays[a].components, (unsigned long long)offs[a]);
        o.put(buf);
    }
    std::snprintf(buf, sizeof buf,
                  "      </PointData>\n      <Points>\n        <DataArray type=\"Float32\" Name=\"Points\" "
                  "NumberOfComponents=\"3\" format=\"appended\" offset=\"%llu\"/>\n      </Points>\n      <Cells>\n",
                  (unsigned long long)off_pts);
    o.put(buf);
    std::snprintf(buf, sizeof buf,
                  "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"%llu\"/>\n"
                  "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"%llu\"/>\n"
                  "        <DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"%llu\"/>\n",
                  (unsigned long long)off_con, (unsigned long long)off_ofs, (unsigned long long)off_typ);
    o.put(buf);
    o.put("      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n   _");
    for (size_t a = 0; a < narrays; ++a) o.raw(arrays[a].data, n * arrays[a].components * sizeof(double));
    o.raw(xyz, n * 3 * sizeof(float));
    {
        std::vector<int64_t> v(n);
        for (size_t i = 0; i < n; ++i) v[i] = (int64_t)i;
        o.raw(v.data(), n * sizeof(int64_t));
        for (size_t i = 0; i < n; ++i) v[i] = (int64_t)i + 1;
        o.raw(v.data(), n * sizeof(int64_t));
    }
    {
        std::vector<uint8_t> t(n, 1);   // VTK_VERTEX
        o.raw(t.data(), n);
    }
    o.put("\n  </AppendedData>\n</VTKFile>\n");
    const bool closed = std::fclose(f) == 0;
    if (!o.ok || !closed) return fail(LBM_ERR_IO, "writing %s failed", path);
    return LBM_OK;
}
