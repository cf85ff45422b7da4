// io.cpp -- the reference's matrix and supernode file formats (utils.cpp:9-109), read and
// written on the host.
//
//   .matrix  binary: int32 n, uint64 nz, int32 col[nz], uint64 row_ptr[n+1], f64 val[nz]
//            (utils.cpp:17-31), CSR with the diagonal first;
//   .txt     text: n nz, then val[nz], col[nz], row_ptr[n+1] (utils.cpp:61-76);
//   .mtx     MatrixMarket coordinate entries of a lower-triangular factor in column order, read
//            as the CSR of its transpose (upper, diagonal first): entry (i, j, v) becomes column
//            i-1 of row j-1 (utils.cpp:32-60); '%' lines are skipped;
//   .snodes  binary: int32 sn, int32 snodes[sn+1] (utils.cpp:89-98); .txt: sn, then the array
//            (utils.cpp:99-105).
// The reference exits or prints on failure; these return a negative sptrsv_status
// (SPTRSV_ERR_IO for an unreadable or malformed file, SPTRSV_ERR_INVALID_ARG for an unknown
// extension).  Arrays are malloc'd and released with sptrsv_io_free.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include "../../include/sptrsv_gb300.h"

namespace {

std::string ext_of(const char* path) {
    const std::string p(path);
    const size_t d = p.find_last_of('.');
    return d == std::string::npos ? std::string() : p.substr(d + 1);
}

template <typename T>
T* alloc_n(size_t count) {
    return (T*)std::malloc(sizeof(T) * (count ? count : 1));
}

bool read_exact(FILE* f, void* p, size_t bytes) { return bytes == 0 || std::fread(p, 1, bytes, f) == bytes; }

}  // namespace

extern "C" {

SPTRSV_API void sptrsv_io_free(void* p) { std::free(p); }

SPTRSV_API int sptrsv_read_csr(const char* path, int* n_out, int64_t* nnz_out, int64_t** row_ptr_out, int** col_out,
                               double** val_out) {
    if (!path || !n_out || !nnz_out || !row_ptr_out || !col_out || !val_out) return SPTRSV_ERR_INVALID_ARG;
    *row_ptr_out = nullptr;
    *col_out = nullptr;
    *val_out = nullptr;
    const std::string ext = ext_of(path);
    int n = 0;
    uint64_t nz = 0;
    int64_t* rp = nullptr;
    int* col = nullptr;
    double* val = nullptr;
    auto bad = [&]() {
        std::free(rp);
        std::free(col);
        std::free(val);
        return SPTRSV_ERR_IO;
    };
    if (ext == "matrix") {
        FILE* f = std::fopen(path, "rb");
        if (!f) return SPTRSV_ERR_IO;
        bool ok = read_exact(f, &n, sizeof(int)) && read_exact(f, &nz, sizeof(uint64_t)) && n > 0 &&
                  nz < (1ull << 40);
        if (ok) {
            rp = alloc_n<int64_t>((size_t)n + 1);
            col = alloc_n<int>(nz);
            val = alloc_n<double>(nz);
            ok = rp && col && val && read_exact(f, col, sizeof(int) * nz) &&
                 read_exact(f, rp, sizeof(uint64_t) * ((size_t)n + 1)) && read_exact(f, val, sizeof(double) * nz);
        }
        std::fclose(f);
        if (!ok) return bad();
    } else if (ext == "txt") {
        std::ifstream in(path);
        if (!(in >> n >> nz) || n <= 0) return SPTRSV_ERR_IO;
        rp = alloc_n<int64_t>((size_t)n + 1);
        col = alloc_n<int>(nz);
        val = alloc_n<double>(nz);
        if (!rp || !col || !val) return bad();
        for (uint64_t i = 0; i < nz; ++i)
            if (!(in >> val[i])) return bad();
        for (uint64_t i = 0; i < nz; ++i)
            if (!(in >> col[i])) return bad();
        for (int i = 0; i <= n; ++i)
            if (!(in >> rp[i])) return bad();
    } else if (ext == "mtx") {
        std::ifstream in(path);
        std::string line;
        int rows = 0, cols = 0;
        while (std::getline(in, line)) {
            if (line.empty() || line[0] == '%') continue;
            std::istringstream hs(line);
            if (!(hs >> rows >> cols >> nz)) return SPTRSV_ERR_IO;
            break;
        }
        if (rows <= 0 || rows != cols) return SPTRSV_ERR_IO;
        n = rows;
        rp = alloc_n<int64_t>((size_t)n + 1);
        col = alloc_n<int>(nz);
        val = alloc_n<double>(nz);
        if (!rp || !col || !val) return bad();
        std::vector<int64_t> count((size_t)n + 1, 0);
        int prev = 0;
        for (uint64_t e = 0; e < nz; ++e) {
            int i, j;
            if (!(in >> i >> j >> val[e]) || i < 1 || i > n || j < 1 || j > n || j < prev) return bad();
            col[e] = i - 1;  // the entry's row becomes the column of row j-1 of the transpose
            ++count[j];
            prev = j;
        }
        rp[0] = 0;
        for (int r = 0; r < n; ++r) rp[r + 1] = rp[r] + count[r + 1];
    } else {
        return SPTRSV_ERR_INVALID_ARG;
    }
    if (rp[0] != 0 || (uint64_t)rp[n] != nz) return bad();
    *n_out = n;
    *nnz_out = (int64_t)nz;
    *row_ptr_out = rp;
    *col_out = col;
    *val_out = val;
    return 0;
}

SPTRSV_API int sptrsv_write_csr(const char* path, int n, int64_t nnz, const int64_t* row_ptr, const int* col,
                                const double* val) {
    if (!path || n <= 0 || nnz < 0 || !row_ptr || !col || !val) return SPTRSV_ERR_INVALID_ARG;
    const std::string ext = ext_of(path);
    if (ext == "matrix") {
        FILE* f = std::fopen(path, "wb");
        if (!f) return SPTRSV_ERR_IO;
        const uint64_t nz = (uint64_t)nnz;
        bool ok = std::fwrite(&n, sizeof(int), 1, f) == 1 && std::fwrite(&nz, sizeof(uint64_t), 1, f) == 1 &&
                  std::fwrite(col, sizeof(int), nz, f) == nz &&
                  std::fwrite(row_ptr, sizeof(uint64_t), (size_t)n + 1, f) == (size_t)n + 1 &&
                  std::fwrite(val, sizeof(double), nz, f) == nz;
        ok = (std::fclose(f) == 0) && ok;
        return ok ? 0 : SPTRSV_ERR_IO;
    }
    if (ext == "txt") {
        FILE* f = std::fopen(path, "w");
        if (!f) return SPTRSV_ERR_IO;
        std::fprintf(f, "%d %lld\n", n, (long long)nnz);
        for (int64_t i = 0; i < nnz; ++i) std::fprintf(f, "%.17g\n", val[i]);
        for (int64_t i = 0; i < nnz; ++i) std::fprintf(f, "%d\n", col[i]);
        for (int i = 0; i <= n; ++i) std::fprintf(f, "%lld\n", (long long)row_ptr[i]);
        return std::fclose(f) == 0 ? 0 : SPTRSV_ERR_IO;
    }
    return SPTRSV_ERR_INVALID_ARG;
}

SPTRSV_API int sptrsv_read_snodes(const char* path, int* sn_out, int** snodes_out) {
    if (!path || !sn_out || !snodes_out) return SPTRSV_ERR_INVALID_ARG;
    *snodes_out = nullptr;
    const std::string ext = ext_of(path);
    int sn = 0;
    int* s = nullptr;
    if (ext == "snodes") {
        FILE* f = std::fopen(path, "rb");
        if (!f) return SPTRSV_ERR_IO;
        bool ok = read_exact(f, &sn, sizeof(int)) && sn > 0;
        if (ok) {
            s = alloc_n<int>((size_t)sn + 1);
            ok = s && read_exact(f, s, sizeof(int) * ((size_t)sn + 1));
        }
        std::fclose(f);
        if (!ok) {
            std::free(s);
            return SPTRSV_ERR_IO;
        }
    } else if (ext == "txt") {
        std::ifstream in(path);
        if (!(in >> sn) || sn <= 0) return SPTRSV_ERR_IO;
        s = alloc_n<int>((size_t)sn + 1);
        for (int i = 0; i <= sn; ++i)
            if (!(in >> s[i])) {
                std::free(s);
                return SPTRSV_ERR_IO;
            }
    } else {
        return SPTRSV_ERR_INVALID_ARG;
    }
    *sn_out = sn;
    *snodes_out = s;
    return 0;
}

SPTRSV_API int sptrsv_write_snodes(const char* path, int sn, const int* snodes) {
    if (!path || sn <= 0 || !snodes) return SPTRSV_ERR_INVALID_ARG;
    const std::string ext = ext_of(path);
    if (ext == "snodes") {
        FILE* f = std::fopen(path, "wb");
        if (!f) return SPTRSV_ERR_IO;
        bool ok = std::fwrite(&sn, sizeof(int), 1, f) == 1 &&
                  std::fwrite(snodes, sizeof(int), (size_t)sn + 1, f) == (size_t)sn + 1;
        ok = (std::fclose(f) == 0) && ok;
        return ok ? 0 : SPTRSV_ERR_IO;
    }
    if (ext == "txt") {
        FILE* f = std::fopen(path, "w");
        if (!f) return SPTRSV_ERR_IO;
        std::fprintf(f, "%d\n", sn);
        for (int i = 0; i <= sn; ++i) std::fprintf(f, "%d\n", snodes[i]);
        return std::fclose(f) == 0 ? 0 : SPTRSV_ERR_IO;
    }
    return SPTRSV_ERR_INVALID_ARG;
}

}  // extern "C"
