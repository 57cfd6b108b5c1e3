// STL input/output and error plumbing of the C ABI (host C++).
//
// The ASCII reader follows the facet grammar of Reader::readSTLASCII
// (GeometryReader.cpp:33-117) line for line, including its recovery rules:
// a facet is kept only when the "facet normal", "outer loop", three "vertex",
// "endloop" and "endfacet" lines parse in sequence; a vertex line that fails
// to parse ends the vertex loop and the following line is then tested as
// "endloop"; corner values persist from the previous facet.  Decimal numbers
// are converted with strtod, which rounds correctly like the reference's
// istream >> double; tokens istream rejects (nan, inf, out of range) are
// rejected here too.
#include <algorithm>
#include <cerrno>
#include <new>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "internal.h"

namespace lbm {

static thread_local std::string g_last_error;

lbm_status fail(lbm_status s, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

void clear_error() { g_last_error.clear(); }

lbm_status to_c_array(const TriVec& v, lbm_tri** out, size_t* n) {
    *out = nullptr;
    *n = 0;
    void* p = std::malloc(sizeof(lbm_tri) * (v.empty() ? 1 : v.size()));
    if (!p) return fail(LBM_ERR_NOMEM, "out of host memory for %zu triangles", v.size());
    if (!v.empty()) std::memcpy(p, v.data(), sizeof(lbm_tri) * v.size());
    *out = (lbm_tri*)p;
    *n = v.size();
    return LBM_OK;
}

namespace {

// Whitespace tokenizer over one line with istream-like failure semantics.
struct Tokens {
    const char* p;
    bool failed = false;
    explicit Tokens(const std::string& s) : p(s.c_str()) {}
    bool word(std::string& out) {
        if (failed) return false;
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) { failed = true; return false; }
        const char* b = p;
        while (*p && !std::isspace((unsigned char)*p)) ++p;
        out.assign(b, p);
        return true;
    }
    bool number(double& out) {
        if (failed) return false;
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) { failed = true; return false; }
        // istream >> double accepts [sign] digits [. digits] [e [sign] digits]
        const char* b = p;
        const char* q = p;
        if (*q == '+' || *q == '-') ++q;
        bool digits = false;
        while (std::isdigit((unsigned char)*q)) { ++q; digits = true; }
        if (*q == '.') { ++q; while (std::isdigit((unsigned char)*q)) { ++q; digits = true; } }
        if (!digits) { failed = true; return false; }
        if (*q == 'e' || *q == 'E') {
            const char* r = q + 1;
            if (*r == '+' || *r == '-') ++r;
            if (std::isdigit((unsigned char)*r)) { while (std::isdigit((unsigned char)*r)) ++r; q = r; }
        }
        std::string tok(b, q);
        errno = 0;
        double v = std::strtod(tok.c_str(), nullptr);
        if (errno == ERANGE && std::isinf(v)) { failed = true; return false; }
        out = v;
        p = q;
        return true;
    }
};

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" {

const char* lbm_last_error(void) { return g_last_error.c_str(); }

const char* lbm_status_string(lbm_status s) {
    switch (s) {
        case LBM_OK: return "LBM_OK";
        case LBM_ERR_IO: return "LBM_ERR_IO";
        case LBM_ERR_PARSE: return "LBM_ERR_PARSE";
        case LBM_ERR_NOMEM: return "LBM_ERR_NOMEM";
        case LBM_ERR_CUDA: return "LBM_ERR_CUDA";
        case LBM_ERR_DIVERGED: return "LBM_ERR_DIVERGED";
        case LBM_ERR_TIMEOUT: return "LBM_ERR_TIMEOUT";
        case LBM_ERR_ARG: return "LBM_ERR_ARG";
        case LBM_ERR_STATE: return "LBM_ERR_STATE";
        case LBM_ERR_NODEV: return "LBM_ERR_NODEV";
    }
    return "LBM_ERR_UNKNOWN";
}

void lbm_free(void* p) { std::free(p); }
int lbm_abi_version(void) { return LBM_ABI_VERSION; }

static lbm_status read_ascii(const char* path, lbm_tri** tris, size_t* n);

lbm_status lbm_stl_read_ascii(const char* path, lbm_tri** tris, size_t* n) {
    if (!path || !tris || !n) return fail(LBM_ERR_ARG, "lbm_stl_read_ascii: null argument");
    clear_error();
    try {
        return read_ascii(path, tris, n);
    } catch (const std::bad_alloc&) {               // no exception crosses the C ABI
        return fail(LBM_ERR_NOMEM, "%s: out of host memory", path);
    }
}

static lbm_status read_ascii(const char* path, lbm_tri** tris, size_t* n) {
    std::ifstream file(path);
    if (!file.is_open()) return fail(LBM_ERR_IO, "cannot open file %s", path);
    TriVec out;
    std::string line, facet, normal, outer, loop, vertex, endloop, endfacet;
    double t[12] = {0};
    while (std::getline(file, line)) {
        {
            Tokens tk(line);
            double a, b, c;
            bool ok = tk.word(facet) & tk.word(normal);
            ok = ok && tk.number(a) && tk.number(b) && tk.number(c);
            if (!ok || facet != "facet" || normal != "normal") continue;
            t[9] = a; t[10] = b; t[11] = c;
        }
        if (!std::getline(file, line)) break;
        {
            Tokens tk(line);
            bool ok = tk.word(outer) && tk.word(loop);
            if (!ok || outer != "outer" || loop != "loop") continue;
        }
        for (int i = 0; i < 3; ++i) {
            if (!std::getline(file, line)) line.clear();
            Tokens tk(line);
            double x, y, z;
            bool ok = tk.word(vertex) && tk.number(x) && tk.number(y) && tk.number(z);
            if (!ok || vertex != "vertex") break;
            t[3 * i] = x; t[3 * i + 1] = y; t[3 * i + 2] = z;
        }
        if (!std::getline(file, line)) line.clear();
        {
            Tokens tk(line);
            if (!tk.word(endloop) || endloop != "endloop") continue;
        }
        if (!std::getline(file, line)) line.clear();
        {
            Tokens tk(line);
            if (!tk.word(endfacet) || endfacet != "endfacet") continue;
        }
        lbm_tri tri;
        std::memcpy(&tri, t, sizeof tri);
        out.push_back(tri);
    }
    return to_c_array(out, tris, n);
}

lbm_status lbm_stl_read_binary(const char* path, lbm_tri** tris, size_t* n) {
    if (!path || !tris || !n) return fail(LBM_ERR_ARG, "lbm_stl_read_binary: null argument");
    clear_error();
    std::ifstream file(path, std::ios::binary);
    if (!file) return fail(LBM_ERR_IO, "cannot open file %s", path);
    char header[80];
    uint32_t count = 0;
    if (!file.read(header, 80) || !file.read(reinterpret_cast<char*>(&count), 4))
        return fail(LBM_ERR_PARSE, "%s: truncated binary STL header", path);
    // the facet count is the file's claim: reserve no more than the bytes
    // after the header can hold (a corrupt count must not allocate for it)
    const std::streampos here = file.tellg();
    file.seekg(0, std::ios::end);
    const std::streamoff left = file.tellg() - here;
    file.seekg(here);
    TriVec out;
    try {
        out.reserve(std::min<uint64_t>(count, left > 0 ? (uint64_t)left / 50 : 0));
        for (uint32_t i = 0; i < count; ++i) {
            float v[12];
            uint16_t attr;
            if (!file.read(reinterpret_cast<char*>(v), 48) || !file.read(reinterpret_cast<char*>(&attr), 2))
                return fail(LBM_ERR_PARSE, "%s: truncated at facet %u of %u", path, i, count);
            // normal first in the file; renormalised in float (GeometryReader.cpp:138-141)
            float nx = v[0], ny = v[1], nz = v[2];
            float norm = std::sqrt(nx * nx + ny * ny + nz * nz);
            nx /= norm; ny /= norm; nz /= norm;
            lbm_tri t = {v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], nx, ny, nz};
            out.push_back(t);
        }
    } catch (const std::bad_alloc&) {
        return fail(LBM_ERR_NOMEM, "%s: out of host memory for %u facets", path, count);
    }
    return to_c_array(out, tris, n);
}

lbm_status lbm_stl_write_ascii(const char* path, const lbm_tri* tris, size_t n, const char* name) {
    if (!path || (!tris && n)) return fail(LBM_ERR_ARG, "lbm_stl_write_ascii: null argument");
    clear_error();
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(LBM_ERR_IO, "cannot write %s", path);
    const char* nm = name ? name : "lbm_gb300";
    std::fprintf(f, "solid %s\n", nm);
    for (size_t i = 0; i < n; ++i) {
        const lbm_tri& t = tris[i];
        std::fprintf(f, "facet normal %.17g %.17g %.17g\nouter loop\n", t.nx, t.ny, t.nz);
        std::fprintf(f, "vertex %.17g %.17g %.17g\n", t.x1, t.y1, t.z1);
        std::fprintf(f, "vertex %.17g %.17g %.17g\n", t.x2, t.y2, t.z2);
        std::fprintf(f, "vertex %.17g %.17g %.17g\n", t.x3, t.y3, t.z3);
        std::fprintf(f, "endloop\nendfacet\n");
    }
    std::fprintf(f, "endsolid %s\n", nm);
    bool ok = std::ferror(f) == 0;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? LBM_OK : fail(LBM_ERR_IO, "write error on %s", path);
}

}  // extern "C"
