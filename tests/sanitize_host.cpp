// Host-side code under AddressSanitizer and UndefinedBehaviorSanitizer (test
// infrastructure, built and run by test_sanitize_cpu.py): the library's host
// STL reader and writer on valid, truncated and malformed files, its mesh
// generators and .vtu writer, and the oracle's voxelizer, boundary search and
// FP64 time loop on a small cylinder.  Exits 0 when every check holds; a
// sanitizer finding aborts with its report.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_gb300.h"

extern "C" {
int64_t orc_read_stl_ascii(const char* path, double** tris_out);
void orc_free(void* p);
void orc_bbox(const double* tris, int64_t n, double bbox[6], int dims[3], double spacing);
int orc_voxelize(const double* tris, int64_t n, const double bbox[6], double spacing, const int dims[3], int binned,
                 uint8_t* flags);
int64_t orc_boundary_points(const uint8_t* flags, const int dims[3], int64_t* out, int64_t cap);
void* orc_sim_create(int Q, const int dims[3], const int8_t* role, int nlists, const int* kinds,
                     const double* list_rho, double tau);
void orc_sim_destroy(void* h);
int64_t orc_sim_nodes(void* h);
void orc_sim_step(void* h, int nsteps);
void orc_sim_get(void* h, double* f, double* rho, double* u);
}

static int failures = 0;
#define CHECK(c)                                                            \
    do {                                                                    \
        if (!(c)) {                                                         \
            std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #c); \
            ++failures;                                                     \
        }                                                                   \
    } while (0)

static std::string slurp(const std::string& p) {
    std::string s;
    FILE* f = std::fopen(p.c_str(), "rb");
    if (!f) return s;
    char buf[4096];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, k);
    std::fclose(f);
    return s;
}
static void spill(const std::string& p, const std::string& s) {
    FILE* f = std::fopen(p.c_str(), "wb");
    if (!f) return;
    std::fwrite(s.data(), 1, s.size(), f);
    std::fclose(f);
}

// Reads a file with both host readers; any status is fine, a crash is not.
static void read_any(const std::string& p) {
    lbm_tri* t = nullptr;
    size_t n = 0;
    if (lbm_stl_read_ascii(p.c_str(), &t, &n) == LBM_OK) lbm_free(t);
    t = nullptr;
    if (lbm_stl_read_binary(p.c_str(), &t, &n) == LBM_OK) lbm_free(t);
    double* o = nullptr;
    if (orc_read_stl_ascii(p.c_str(), &o) >= 0 && o) orc_free(o);
}

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    // 1. a cylinder from the generator, written and read back (ASCII)
    lbm_tri* tris = nullptr;
    size_t nt = 0;
    const double c[3] = {9.3, 13.1, 9.7};
    CHECK(lbm_synth_cylinder(6.0, 20.0, 24, 1, c, &tris, &nt) == LBM_OK && nt > 0);
    const std::string asc = dir + "/cyl.stl";
    CHECK(lbm_stl_write_ascii(asc.c_str(), tris, nt, "cyl") == LBM_OK);
    lbm_tri* back = nullptr;
    size_t nb = 0;
    CHECK(lbm_stl_read_ascii(asc.c_str(), &back, &nb) == LBM_OK && nb == nt);
    if (back) lbm_free(back);

    // 2. malformed ASCII: every prefix length step, garbage, empty, lone keywords
    const std::string text = slurp(asc);
    for (size_t cut = 0; cut < text.size(); cut += 97) {
        spill(dir + "/cut.stl", text.substr(0, cut));
        read_any(dir + "/cut.stl");
    }
    std::string garbage;
    for (int i = 0; i < 5000; ++i) garbage.push_back((char)((i * 7919 + 13) & 0xff));
    spill(dir + "/garbage.stl", garbage);
    read_any(dir + "/garbage.stl");
    spill(dir + "/empty.stl", "");
    read_any(dir + "/empty.stl");
    spill(dir + "/keywords.stl", "solid x\nfacet normal\nouter loop\nvertex 1 2\nendloop\nendfacet\nfacet normal 1e999 -nan 0\n");
    read_any(dir + "/keywords.stl");

    // 3. binary STL written by hand (80-byte header, count, 50 bytes a facet), read back, then truncated
    std::string bin(80, ' ');
    const uint32_t cnt = (uint32_t)nt;
    bin.append((const char*)&cnt, 4);
    for (size_t t = 0; t < nt; ++t) {
        const double* T = &tris[t].x1;
        float v[12];
        // normal, then the three vertices (lbm_tri stores the vertices first, the normal last)
        for (int a = 0; a < 3; ++a) v[a] = (float)T[9 + a];
        for (int a = 0; a < 9; ++a) v[3 + a] = (float)T[a];
        bin.append((const char*)v, sizeof v);
        bin.append(2, '\0');
    }
    const std::string binp = dir + "/cyl_bin.stl";
    spill(binp, bin);
    lbm_tri* bt = nullptr;
    size_t bn = 0;
    CHECK(lbm_stl_read_binary(binp.c_str(), &bt, &bn) == LBM_OK && bn == nt);
    if (bt) lbm_free(bt);
    for (size_t cut = 0; cut < bin.size(); cut += 61) {
        spill(dir + "/bcut.stl", bin.substr(0, cut));
        read_any(dir + "/bcut.stl");
    }
    std::string big = bin;
    const uint32_t huge = 0x7fffffffu;
    std::memcpy(&big[80], &huge, 4);
    spill(dir + "/bhuge.stl", big);
    read_any(dir + "/bhuge.stl");

    // 4. capsule mesh and .vtu writer
    const double seg[20] = {4, 4, 4, 14, 12, 6, 2.5, -1, 0, 0, 14, 12, 6, 14, 20, 14, 2.0, 1, 19.5, 1};
    const double lo[3] = {0, 0, 0}, hi[3] = {20, 24, 20};
    lbm_tri* ct = nullptr;
    size_t cn = 0;
    CHECK(lbm_synth_capsules(seg, 2, lo, hi, 1.1, 7, &ct, &cn) == LBM_OK && cn > 0);
    if (ct) lbm_free(ct);
    std::vector<float> xyz(30);
    std::vector<double> a1(10), a3(30);
    for (int i = 0; i < 30; ++i) { xyz[i] = (float)i; a3[i] = 0.5 * i; }
    for (int i = 0; i < 10; ++i) a1[i] = i;
    const lbm_vtu_array arrs[2] = {{"Density", 1, 0, a1.data()}, {"Velocity", 3, 0, a3.data()}};
    CHECK(lbm_vtu_write((dir + "/p.vtu").c_str(), 10, xyz.data(), 2, arrs) == LBM_OK);

    // 5. the oracle on the cylinder: voxelize, boundary points, 6 FP64 steps (walls only)
    std::vector<double> flat(12 * nt);
    std::memcpy(flat.data(), tris, sizeof(double) * 12 * nt);
    double bbox[6];
    int dims[3];
    orc_bbox(flat.data(), (int64_t)nt, bbox, dims, 1.0);
    const size_t np = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<uint8_t> flags(np);
    CHECK(orc_voxelize(flat.data(), (int64_t)nt, bbox, 1.0, dims, 1, flags.data()) == 0);
    size_t nfl = 0;
    for (uint8_t f : flags) nfl += f != 0;
    CHECK(nfl > 100);
    const int64_t nbd = orc_boundary_points(flags.data(), dims, nullptr, 0);
    std::vector<int64_t> bidx((size_t)(nbd > 0 ? nbd : 1));
    CHECK(orc_boundary_points(flags.data(), dims, bidx.data(), nbd) == nbd);
    std::vector<int8_t> role(np, -1);
    for (size_t p = 0; p < np; ++p) if (flags[p]) role[p] = 0;
    for (int64_t b = 0; b < nbd; ++b) role[(size_t)bidx[b]] = 1;
    std::vector<int> kinds(64, 0);
    std::vector<double> rho(64, 1.0);
    void* sim = orc_sim_create(19, dims, role.data(), 64, kinds.data(), rho.data(), 0.8);
    const int64_t nn = orc_sim_nodes(sim);
    CHECK(nn == (int64_t)nfl);
    orc_sim_step(sim, 6);
    std::vector<double> f((size_t)nn * 19), r((size_t)nn), u((size_t)nn * 3);
    orc_sim_get(sim, f.data(), r.data(), u.data());
    double mass = 0;
    for (double v : r) { CHECK(std::isfinite(v)); mass += v; }
    CHECK(std::fabs(mass / (double)nn - 1.0) < 1e-9);     // closed walls, fluid at rest: mass stays
    orc_sim_destroy(sim);
    lbm_free(tris);
    if (failures) std::fprintf(stderr, "%d check(s) failed\n", failures);
    else std::printf("sanitized host run ok: %zu triangles, %zu fluid points\n", nt, nfl);
    return failures ? 1 : 0;
}
