// ASCII STL parsing on the GPU (lbm_stl_read_ascii_device).
//
// Same result as lbm_stl_read_ascii (stl_io.cpp), which follows the facet
// grammar of Reader::readSTLASCII (GeometryReader.cpp:33-117): the file is
// copied to the device once, every line start is found by a compaction of
// the newline positions, every line whose first word is "facet" starts a
// candidate facet, and one thread per candidate checks the seven lines
//   facet normal nx ny nz / outer loop / vertex x y z (3x) / endloop / endfacet
// with the host tokenizer's rules (words are maximal non-space runs, numbers
// the longest prefix of [sign] digits [. digits] [e [sign] digits]) and
// converts the twelve numbers exactly (stl_number.h).  A file in that
// canonical form gives the triangles in file order.  Anything else -- a
// candidate that does not parse, a number outside the exact converter's
// scope, a NUL byte -- makes the reader parse the whole file with the host
// grammar instead (its recovery rules for broken facets depend on the lines
// before them), and *on_device reports which path produced the result.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <cuda_runtime.h>

#include "device.cuh"
#include "internal.h"
#include "scan.cuh"
#include "stl_number.h"

#define LBM_TRY(x)                      \
    do {                                \
        lbm_status s_ = (x);            \
        if (s_ != LBM_OK) return s_;    \
    } while (0)

namespace lbm {
namespace {

__device__ __forceinline__ bool is_ws(char c) {
    return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f' || c == '\n';
}

// next word of [p, e): returns its end and sets *b to its start; nullptr
// when the line has no further word
__device__ const char* next_word(const char* p, const char* e, const char** b) {
    while (p < e && is_ws(*p)) ++p;
    if (p >= e) return nullptr;
    *b = p;
    while (p < e && !is_ws(*p)) ++p;
    return p;
}

__device__ bool word_eq(const char* b, const char* w_end, const char* lit) {
    const char* p = b;
    while (*lit) {
        if (p >= w_end || *p != *lit) return false;
        ++p;
        ++lit;
    }
    return p == w_end;
}

// line j: [t + ls[j], t + line end) without its newline
struct Lines {
    const char* t;
    int64_t L;
    const int64_t* ls;
    int64_t nl;
    __device__ void get(int64_t j, const char** b, const char** e) const {
        const int64_t s = ls[j];
        int64_t end = j + 1 < nl ? ls[j + 1] - 1 : L;
        if (j + 1 >= nl && end > s && t[end - 1] == '\n') --end;
        *b = t + s;
        *e = t + (end < s ? s : end);
    }
};

__global__ void k_line_starts(const char* __restrict__ t, int64_t L, uint8_t* __restrict__ f) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L; i += (int64_t)gridDim.x * blockDim.x)
        f[i] = (i == 0 || t[i - 1] == '\n') ? 1 : 0;
}

__global__ void k_facet_lines(Lines ln, uint8_t* __restrict__ f) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ln.nl; j += (int64_t)gridDim.x * blockDim.x) {
        const char *b, *e, *wb;
        ln.get(j, &b, &e);
        const char* we = next_word(b, e, &wb);
        f[j] = (we && word_eq(wb, we, "facet")) ? 1 : 0;
    }
}

// status bits
constexpr int kBadStructure = 1;
constexpr int kInexact = 2;

__device__ bool numbers(const char* p, const char* e, int k, double* out, int* status) {
    for (int i = 0; i < k; ++i) {
        bool exact = false;
        p = stlnum::parse_number(p, e, out + i, &exact);
        if (!p) return false;
        if (!exact) *status |= kInexact;
    }
    return true;
}

__global__ void k_facets(Lines ln, const int64_t* __restrict__ fl, int64_t nf, lbm_tri* __restrict__ out,
                         int32_t* __restrict__ status) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nf; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = fl[k];
        int st = 0;
        double v[12];
        if (j + 6 >= ln.nl) {
            st = kBadStructure;
        } else {
            const char *b, *e, *wb, *we;
            // facet normal nx ny nz
            ln.get(j, &b, &e);
            we = next_word(b, e, &wb);                       // "facet" (the candidate test)
            const char* wb2;
            const char* we2 = next_word(we, e, &wb2);
            if (!we2 || !word_eq(wb2, we2, "normal") || !numbers(we2, e, 3, v + 9, &st)) st |= kBadStructure;
            // outer loop
            ln.get(j + 1, &b, &e);
            we = next_word(b, e, &wb);
            if (!we || !word_eq(wb, we, "outer")) st |= kBadStructure;
            else {
                we2 = next_word(we, e, &wb2);
                if (!we2 || !word_eq(wb2, we2, "loop")) st |= kBadStructure;
            }
            // three vertices
            for (int c = 0; c < 3; ++c) {
                ln.get(j + 2 + c, &b, &e);
                we = next_word(b, e, &wb);
                if (!we || !word_eq(wb, we, "vertex") || !numbers(we, e, 3, v + 3 * c, &st)) st |= kBadStructure;
            }
            ln.get(j + 5, &b, &e);
            we = next_word(b, e, &wb);
            if (!we || !word_eq(wb, we, "endloop")) st |= kBadStructure;
            ln.get(j + 6, &b, &e);
            we = next_word(b, e, &wb);
            if (!we || !word_eq(wb, we, "endfacet")) st |= kBadStructure;
        }
        if (st) {
            atomicOr(status, st);
            continue;
        }
        lbm_tri tri;
        tri.x1 = v[0]; tri.y1 = v[1]; tri.z1 = v[2];
        tri.x2 = v[3]; tri.y2 = v[4]; tri.z2 = v[5];
        tri.x3 = v[6]; tri.y3 = v[7]; tri.z3 = v[8];
        tri.nx = v[9]; tri.ny = v[10]; tri.nz = v[11];
        out[k] = tri;
    }
}

unsigned grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b > 152 * 64) b = 152 * 64;
    return (unsigned)(b > 0 ? b : 1);
}

// device buffers of one parse, released on every path
struct ParseBufs {
    cudaStream_t st = 0;
    char* text = nullptr;
    uint8_t* flags = nullptr;
    int64_t* ls = nullptr;
    int64_t* fl = nullptr;
    lbm_tri* tris = nullptr;
    int32_t* status = nullptr;
    ~ParseBufs() {
        cudaStreamSynchronize(st);         // ls, fl come from the stream-ordered pool: no implicit wait
        cudaFree(text);
        cudaFree(flags);
        cudaFree(ls);
        cudaFree(fl);
        cudaFree(tris);
        cudaFree(status);
    }
};

lbm_status parse_on_device(const char* host_text, int64_t L, cudaStream_t st, lbm_tri** tris, size_t* n,
                           bool* ok) {
    ParseBufs B;
    B.st = st;
    *ok = false;
    if (L == 0) {                           // no lines, no facets
        *tris = (lbm_tri*)std::malloc(sizeof(lbm_tri));
        if (!*tris) return fail(LBM_ERR_NOMEM, "out of host memory");
        *n = 0;
        *ok = true;
        return LBM_OK;
    }
    LBM_CUDA(cudaMalloc(&B.text, (size_t)L));
    LBM_CUDA(cudaMalloc(&B.status, sizeof(int32_t)));
    LBM_CUDA(cudaMemsetAsync(B.status, 0, sizeof(int32_t), st));
    LBM_CUDA(cudaMemcpyAsync(B.text, host_text, (size_t)L, cudaMemcpyHostToDevice, st));
    LBM_CUDA(cudaMalloc(&B.flags, (size_t)L));
    k_line_starts<<<grid_for(L, 256), 256, 0, st>>>(B.text, L, B.flags);
    LBM_CUDA(cudaGetLastError());
    int64_t nl = 0;
    LBM_TRY(scan::compact(B.flags, L, &B.ls, &nl, st));
    Lines ln{B.text, L, B.ls, nl};
    int64_t nf = 0;
    if (nl > 0) {
        k_facet_lines<<<grid_for(nl, 256), 256, 0, st>>>(ln, B.flags);
        LBM_CUDA(cudaGetLastError());
        LBM_TRY(scan::compact(B.flags, nl, &B.fl, &nf, st));
    }
    if (nf > 0) {
        LBM_CUDA(cudaMalloc(&B.tris, sizeof(lbm_tri) * (size_t)nf));
        k_facets<<<grid_for(nf, 128), 128, 0, st>>>(ln, B.fl, nf, B.tris, B.status);
        LBM_CUDA(cudaGetLastError());
    }
    int32_t hst = 0;
    LBM_CUDA(cudaMemcpyAsync(&hst, B.status, sizeof hst, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    if (hst) return LBM_OK;                 // *ok stays false: the host grammar decides
    lbm_tri* out = (lbm_tri*)std::malloc(sizeof(lbm_tri) * (size_t)(nf > 0 ? nf : 1));
    if (!out) return fail(LBM_ERR_NOMEM, "out of host memory for %lld triangles", (long long)nf);
    if (nf > 0) {
        const cudaError_t e = cudaMemcpyAsync(out, B.tris, sizeof(lbm_tri) * (size_t)nf, cudaMemcpyDeviceToHost, st);
        const cudaError_t e2 = e == cudaSuccess ? cudaStreamSynchronize(st) : e;
        if (e2 != cudaSuccess) {
            std::free(out);
            return fail(LBM_ERR_CUDA, "triangle copy: %s", cudaGetErrorString(e2));
        }
    }
    *tris = out;
    *n = (size_t)nf;
    *ok = true;
    return LBM_OK;
}

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" lbm_status lbm_stl_read_ascii_device(const char* path, void* stream, lbm_tri** tris, size_t* n,
                                                int32_t* on_device) {
    if (!path || !tris || !n) return fail(LBM_ERR_ARG, "lbm_stl_read_ascii_device: null argument");
    clear_error();
    *tris = nullptr;
    *n = 0;
    if (on_device) *on_device = 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(LBM_ERR_NODEV, "lbm_stl_read_ascii_device: no CUDA device");
    }
    FILE* fh = std::fopen(path, "rb");
    if (!fh) return fail(LBM_ERR_IO, "cannot open file %s", path);
    std::fseek(fh, 0, SEEK_END);
    const long sz = std::ftell(fh);
    std::fseek(fh, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(fh);
        return fail(LBM_ERR_IO, "cannot size file %s", path);
    }
    // pinned host memory for the copy to the device; ordinary memory when
    // pinning that much fails (the copy is then slower, the result the same)
    char* text = nullptr;
    bool pinned = cudaMallocHost(&text, (size_t)(sz > 0 ? sz : 1)) == cudaSuccess;
    if (!pinned) {
        cudaGetLastError();
        text = (char*)std::malloc((size_t)(sz > 0 ? sz : 1));
        if (!text) {
            std::fclose(fh);
            return fail(LBM_ERR_NOMEM, "cannot hold %ld bytes of %s", sz, path);
        }
    }
    auto release = [&]() {
        if (pinned) cudaFreeHost(text);
        else std::free(text);
    };
    const size_t got = sz > 0 ? std::fread(text, 1, (size_t)sz, fh) : 0;
    std::fclose(fh);
    if (got != (size_t)sz) {
        release();
        return fail(LBM_ERR_IO, "short read of %s", path);
    }
    bool ok = false;
    lbm_status s = LBM_OK;
    // NUL bytes end the host tokenizer's lines early: host grammar
    if (!std::memchr(text, 0, (size_t)sz))
        s = parse_on_device(text, (int64_t)sz, (cudaStream_t)stream, tris, n, &ok);
    release();
    if (s != LBM_OK) return s;
    if (ok) {
        if (on_device) *on_device = 1;
        return LBM_OK;
    }
    return lbm_stl_read_ascii(path, tris, n);
}
