// csr_tool -- loads a matrix file through CSRHost exactly as the matrix_exp
// program does (format detection, validation, exit codes) and writes the
// resulting CSR arrays as raw little-endian files <out>.rowptr (int32),
// <out>.col (int32) and <out>.val (float64). Used by the loader tests.
// csr_tool MATRIX --time instead times the host loader and the upload of its
// CSR into a device context (mexk_context_upload_csr, m = 30):
// "host_load_s=... upload_s=...".
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "matrix_exp_krylov.hpp"

static bool ends_with(const std::string& s, const std::string& suf) {
    return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: csr_tool MATRIX OUT_PREFIX" << std::endl;
        return 2;
    }
    const std::string path = argv[1], out = argv[2];
    const auto t0 = std::chrono::steady_clock::now();
    CSRHost A;
    std::ifstream f(path, std::ios::binary);
    unsigned char h[8] = {0};
    f.read(reinterpret_cast<char*>(h), 8);
    static const unsigned char magic[8] = {'C', 'S', 'R', 0, 0, 0, 0, 1};
    const bool magic_ok = f.gcount() == 8 && std::memcmp(h, magic, 8) == 0;
    if (ends_with(path, ".bincsr") || magic_ok) A.from_binary_csr(path);
    else if (ends_with(path, ".mtx") || ends_with(path, ".mtx.gz")) A.from_matrix_market(path);
    else {
        std::cerr << "Error: Could not detect matrix format for file " << path << std::endl;
        return 1;
    }
    if (out == "--time") {
        const auto t1 = std::chrono::steady_clock::now();
        mexk_context_t ctx = nullptr;
        int rc = mexk_context_create(0, &ctx);
        if (rc == MEXK_OK)
            rc = mexk_context_upload_csr(ctx, A.rows, A.nnz, A.row_ptr.data(), A.col_idx.data(), A.values.data(), 30);
        const auto t2 = std::chrono::steady_clock::now();
        if (ctx) mexk_context_destroy(ctx);
        if (rc != MEXK_OK) {
            std::cerr << "upload failed: " << mexk_last_error_detail() << std::endl;
            return 1;
        }
        std::cout << "host_load_s=" << std::chrono::duration<double>(t1 - t0).count()
                  << " upload_s=" << std::chrono::duration<double>(t2 - t1).count() << std::endl;
        return 0;
    }
    std::ofstream(out + ".rowptr", std::ios::binary)
        .write(reinterpret_cast<const char*>(A.row_ptr.data()), sizeof(int) * A.row_ptr.size());
    std::ofstream(out + ".col", std::ios::binary)
        .write(reinterpret_cast<const char*>(A.col_idx.data()), sizeof(int) * A.col_idx.size());
    std::ofstream(out + ".val", std::ios::binary)
        .write(reinterpret_cast<const char*>(A.values.data()), sizeof(double) * A.values.size());
    std::cout << "rows=" << A.rows << " cols=" << A.cols << " nnz=" << A.nnz << std::endl;
    return 0;
}
