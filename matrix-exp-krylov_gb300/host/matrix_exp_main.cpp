// matrix_exp -- drop-in replacement for the reference's GPU command line
// program (kol-di/matrix-exp-krylov main.cu:2083-2324): same positional
// arguments and flags, defaults, format detection, built-in diagonal test
// matrix, t clamp to 10/max|A_ij|, m default min(30, max(5, n-1)),
// tolerance 1e-6, v = 0.1, OUTPUT_Y_FILE dump and summary lines. It runs on
// one GPU. Extra flags: --precision fp64|mixed (default fp64, the
// reference's arithmetic), --controller reference|search|learned (default
// the reference's heuristic), --window W (symmetric A, either precision:
// orthogonalise against the last W basis vectors), --quiet (no
// [STEP]/[FLOPs] lines), --verbose-h (the reference's per-step
// "H_m column j stored" lines, main.cu:1951) and --host-load. A .bincsr input is loaded straight
// into the device context (mexk_context_load_bincsr: mapped, streamed,
// checked on the device) with the host loader's output and messages;
// --host-load, symmetric_upper files and non-square matrices take the host
// loader (CSRHost::from_binary_csr).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "matrix_exp_krylov.hpp"

namespace {

bool ends_with(const std::string& s, const std::string& suf) {
    return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

bool has_bincsr_magic(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) return false;
    unsigned char h[8] = {0};
    f.read(reinterpret_cast<char*>(h), 8);
    if (!f || f.gcount() != 8) return false;
    static const unsigned char magic[8] = {'C', 'S', 'R', 0, 0, 0, 0, 1};
    return std::memcmp(h, magic, 8) == 0;
}

}  // namespace

int main(int argc, char* argv[]) {
    std::cout << "Starting matrix_exp application." << std::endl;
    bool use_file = false;
    std::string matrix_file;
    int test_size = 1000;
    int m_param = -1;
    int max_restarts_cli = MAX_RESTARTS;
    double t_cli = 1.0;
    int precision = MEXK_PREC_FP64;
    int controller = MEXK_CTRL_REFERENCE;
    int window = 0;
    bool quiet = false;
    bool verbose_h = false;
    bool host_load = false;

    std::vector<std::string> args(argv + 1, argv + argc);
    size_t pos = 0;
    for (size_t i = 0; i < args.size(); ++i) {
        const std::string& a = args[i];
        if (a == "--m" && i + 1 < args.size()) {
            m_param = std::atoi(args[++i].c_str());
            continue;
        }
        if (a == "--max-restarts" && i + 1 < args.size()) {
            max_restarts_cli = std::atoi(args[++i].c_str());
            continue;
        }
        if (a == "--t" && i + 1 < args.size()) {
            t_cli = std::atof(args[++i].c_str());
            continue;
        }
        if (a == "--precision" && i + 1 < args.size()) {
            const std::string v = args[++i];
            if (v == "mixed") precision = MEXK_PREC_MIXED;
            else if (v == "fp64") precision = MEXK_PREC_FP64;
            else {
                std::cerr << "Error: --precision must be fp64 or mixed" << std::endl;
                return EXIT_FAILURE;
            }
            continue;
        }
        if (a == "--controller" && i + 1 < args.size()) {
            const std::string v = args[++i];
            if (v == "reference") controller = MEXK_CTRL_REFERENCE;
            else if (v == "search") controller = MEXK_CTRL_SEARCH;
            else if (v == "learned") controller = MEXK_CTRL_LEARNED;
            else {
                std::cerr << "Error: --controller must be reference, search or learned" << std::endl;
                return EXIT_FAILURE;
            }
            continue;
        }
        if (a == "--window" && i + 1 < args.size()) {
            window = std::atoi(args[++i].c_str());
            continue;
        }
        if (a == "--quiet") {
            quiet = true;
            continue;
        }
        if (a == "--verbose-h") {
            verbose_h = true;
            continue;
        }
        if (a == "--host-load") {
            host_load = true;
            continue;
        }
        if (pos == 0) {
            if (a.find('.') != std::string::npos || a.find('/') != std::string::npos ||
                a.rfind(".mtx") != std::string::npos) {
                use_file = true;
                matrix_file = a;
            } else {
                test_size = std::atoi(a.c_str());
                if (test_size <= 0) {
                    std::cerr << "Error: Matrix size must be a positive integer. Using default size 1000." << std::endl;
                    test_size = 1000;
                }
            }
            ++pos;
        } else if (pos == 1) {
            m_param = std::atoi(a.c_str());
            ++pos;
        } else if (pos == 2) {
            max_restarts_cli = std::atoi(a.c_str());
            ++pos;
        }
    }

    int num_gpus = 0;
    if (mexk_device_count(&num_gpus) != MEXK_OK) {
        std::cerr << "CUDA Error: " << mexk_last_error_detail() << std::endl;
        return EXIT_FAILURE;
    }
    std::cout << "Found " << num_gpus << " GPU(s)" << std::endl;
    if (num_gpus < 1) {
        std::cerr << "No GPUs found!" << std::endl;
        return EXIT_FAILURE;
    }
    const int gpus_used = 1;  // single-device build: one partition

    CSRHost A;
    mexk_context_t loaded_ctx = nullptr;  // .bincsr loaded straight into the device context
    double loaded_max_abs = 0.0;
    if (use_file) {
        std::cout << "Loading matrix from file: " << matrix_file << std::endl;
        const bool is_bin = ends_with(matrix_file, ".bincsr");
        const bool is_mtx = ends_with(matrix_file, ".mtx") || ends_with(matrix_file, ".mtx.gz");
        bool loaded = false;
        if (is_bin || has_bincsr_magic(matrix_file)) {
            mexk_bincsr_info_t info{};
            const bool direct = !host_load && mexk_bincsr_probe(matrix_file.c_str(), &info) == MEXK_OK &&
                                (info.flags & 4u) == 0 && info.rows == info.cols && info.rows > 1;
            if (direct) {
                const int rows = static_cast<int>(info.rows);
                int m_alloc = m_param > 0 ? m_param : std::min(30, std::max(5, rows - 1));
                m_alloc = std::max(1, std::min(std::min(m_alloc, rows - 1), MEXK_M_MAX));
                int rc = mexk_context_create(0, &loaded_ctx);
                if (rc == MEXK_OK) rc = mexk_context_load_bincsr(loaded_ctx, matrix_file.c_str(), m_alloc, &info);
                if (info.checks_passed >= 3)  // the host loader prints this line before the row checks
                    std::cout << "Binary CSR header: version=1 flags=0x" << std::hex << info.flags << std::dec
                              << " index_dtype=" << (info.index_dtype == 1 ? "u32" : "u64")
                              << " value_dtype=" << (info.value_dtype == 1 ? "f32" : "f64")
                              << " symmetric_upper=no" << std::endl;
                if (rc != MEXK_OK) {
                    std::cerr << mexk_last_error_detail() << std::endl;
                    if (loaded_ctx) mexk_context_destroy(loaded_ctx);
                    return EXIT_FAILURE;
                }
                A.rows = rows;
                A.cols = static_cast<int>(info.cols);
                A.nnz = info.nnz;
                loaded_max_abs = info.max_abs;
            } else {
                A.from_binary_csr(matrix_file);
            }
            loaded = true;
            std::cout << "Detected Binary CSR v1 input" << std::endl;
        } else if (is_mtx) {
            A.from_matrix_market(matrix_file);
            loaded = true;
            std::cout << "Detected MatrixMarket input" << std::endl;
        }
        if (!loaded) {
            std::cerr << "Error: Could not detect matrix format for file " << matrix_file
                      << ". Supported: .bincsr, .mtx, .mtx.gz" << std::endl;
            return EXIT_FAILURE;
        }
        std::cout << "Loaded matrix: " << A.rows << "x" << A.cols << " with " << A.nnz << " non-zeros" << std::endl;
    } else {
        std::cout << "Matrix size (generated): " << test_size << std::endl;
        A.rows = A.cols = test_size;
        A.nnz = test_size;
        A.row_ptr.resize(static_cast<size_t>(test_size) + 1);
        A.col_idx.resize(static_cast<size_t>(test_size));
        A.values.resize(static_cast<size_t>(test_size));
        for (int i = 0; i < test_size; ++i) {
            A.row_ptr[i] = i;
            A.col_idx[i] = i;
            A.values[i] = 1.0 + static_cast<double>(i) / A.rows;
        }
        A.row_ptr[test_size] = test_size;
        std::cout << "Created test matrix: " << A.rows << "x" << A.cols << " with " << A.nnz << " non-zeros"
                  << std::endl;
    }

    // t clamp: keep t*max|A_ij| <= 10 (main.cu:2227-2242).
    double max_abs = loaded_max_abs;
    for (double v : A.values) max_abs = std::max(max_abs, std::abs(v));
    if (max_abs <= 0.0) max_abs = 1.0;
    double t_safe = t_cli;
    const double t_limit = 10.0 / max_abs;
    if (t_safe > t_limit) {
        std::cout << "[WARN] Requested t=" << t_safe << " is large for max|A|=" << max_abs << ". Clamping t to "
                  << t_limit << " to avoid overflow." << std::endl;
        t_safe = t_limit;
    }

    std::vector<CSRHost> parts;
    std::vector<CSRHost::GhostMap> ghosts(gpus_used);
    if (!loaded_ctx) {
        parts = A.partition_rows(gpus_used);
        for (int i = 0; i < gpus_used; ++i) ghosts[i] = A.build_owner_ghost_maps(parts, i, gpus_used);
    }
    std::cout << "Partitioned matrix across " << gpus_used << " GPUs" << std::endl;
    if (!loaded_ctx) validate_ghost_maps(ghosts, gpus_used);

    int m_val = m_param;
    if (m_val <= 0) m_val = std::min(30, std::max(5, A.rows - 1));
    m_val = std::max(1, std::min(m_val, A.rows - 1));
    ArnoldiParams params(m_val, t_safe, 1e-6, max_restarts_cli, true);
    std::cout << "Arnoldi params: m=" << params.m << " t=" << params.t << " tol=" << params.tol
              << " max_restarts=" << params.max_restarts << std::endl;

    ArnoldiRunner runner(gpus_used, params, A.rows, A.cols, A.nnz);
    runner.precision = precision;
    runner.controller = controller;
    runner.ortho_window = window;
    runner.verbose = !quiet;
    runner.log_h_columns = verbose_h;
    if (loaded_ctx)
        runner.init_from_context(loaded_ctx, 0);
    else
        runner.init_all_devices(parts, std::vector<int>{0}, ghosts);
    std::vector<double> v(static_cast<size_t>(A.rows), 0.1);
    std::vector<double> y(static_cast<size_t>(A.rows), 0.0);
    runner.compute_expmv(v, y);

    if (const char* out = std::getenv("OUTPUT_Y_FILE"); out && out[0] != '\0') {
        std::ofstream ofs(out);
        if (!ofs) {
            std::cerr << "Error: could not open OUTPUT_Y_FILE=" << out << " for writing" << std::endl;
            return EXIT_FAILURE;
        }
        ofs.setf(std::ios::scientific);
        ofs.precision(16);
        for (double x : y) ofs << x << "\n";
        std::cout << "Saved y to " << out << std::endl;
    }
    std::cout << "Computation completed. Sample results:" << std::endl;
    for (int i = 0; i < std::min(10, static_cast<int>(y.size())); ++i)
        std::cout << "y[" << i << "] = " << y[i] << std::endl;
    std::cout << "Arnoldi summary: m=" << m_val << ", max_restarts=" << max_restarts_cli
              << ", restarts_done=" << runner.restarts_done << ", converged=" << (runner.converged ? "yes" : "no")
              << ", residual=" << runner.last_residual << std::endl;
    runner.destroy();
    return 0;
}
