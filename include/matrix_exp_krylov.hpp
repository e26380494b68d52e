// matrix_exp_krylov.hpp -- drop-in C++ API of the GB300 exp(t*A)*v solver.
//
// Same type names, members, constructor signatures and call order as the
// reference's single-file program (kol-di/matrix-exp-krylov main.cu):
//   CSRHost            main.cu:86-692   loaders, row partitioning, ghost maps
//   ArnoldiParams      main.cu:1221-1230
//   ExpmvMode          main.cu:1232-1235
//   TimeSteppingParams main.cu:1237-1250
//   DeviceContext      main.cu:747-1125
//   ArnoldiRunner      main.cu:1253-2081
// A program written against those classes compiles against this header and
// links libmexk_host.so + libmexk.so. Underneath, every device operation goes
// through the C ABI in mexk.h (no cuSPARSE, cuBLAS, NCCL or Eigen).
//
// One device: the reference's row partitions are concatenated back into one
// matrix on device_ids[0]; ghost maps are accepted and ignored (a single
// partition has none). Errors keep the reference's behaviour: a message on
// stderr and exit(EXIT_FAILURE).
#pragma once

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "mexk.h"

// main.cu:81-82
const double ARNOLDI_TOL = 1e-8;
const int MAX_RESTARTS = 10;

struct CSRHost {
    int rows;
    int cols;
    long long nnz;
    std::vector<int> row_ptr;
    std::vector<int> col_idx;
    std::vector<double> values;

    CSRHost() : rows(0), cols(0), nnz(0) {}

    // Coordinate real/pattern, general/symmetric MatrixMarket; entries are
    // sorted and duplicates summed (main.cu:97-245).
    void from_matrix_market(const std::string& filename);
    // Binary CSR v1 with the reference's validation (main.cu:265-523).
    void from_binary_csr(const std::string& filename);
    // 1D row blocks, remainder rows to the first blocks (main.cu:526-562).
    std::vector<CSRHost> partition_rows(int num_gpus) const;

    // Halo description for row-parallel SpMV (main.cu:568-585). Built for
    // API compatibility; a single device needs none.
    struct GhostMap {
        std::vector<int> ghost_indices;
        std::vector<int> ghost_owners;
        std::map<int, std::vector<int>> owner_to_consumer_map;
        std::map<int, std::vector<int>> consumer_to_owner_map;
        std::vector<int> send_offsets;
        std::vector<int> recv_offsets;
        std::vector<int> send_counts;
        std::vector<int> recv_counts;
        std::vector<int> outgoing_global_col_indices;
        std::vector<int> incoming_global_col_indices;
        std::map<int, std::pair<size_t, size_t>> outgoing_peer_info;
        std::map<int, std::pair<size_t, size_t>> incoming_peer_info;
        size_t total_recv_size = 0;
        size_t total_send_size = 0;
    };
    GhostMap build_owner_ghost_maps(const std::vector<CSRHost>& partitions, int my_gpu_id, int num_gpus) const;
};

// main.cu:695-744: SEND and RECEIVE plans must agree between every pair.
void validate_ghost_maps(const std::vector<CSRHost::GhostMap>& ghost_maps, int num_gpus);

struct ArnoldiParams {
    int m;
    double t;
    double tol;
    int max_restarts;
    bool reorthogonalize;

    ArnoldiParams(int m_val = 100, double t_val = 1.0, double tol_val = ARNOLDI_TOL,
                  int max_restarts_val = MAX_RESTARTS, bool reortho = true)
        : m(m_val), t(t_val), tol(tol_val), max_restarts(max_restarts_val), reorthogonalize(reortho) {}
};

enum class ExpmvMode { AdaptiveTimeStepping, RestartedKrylov };

struct TimeSteppingParams {
    double dt_init{0.0};
    double dt_min{0.0};
    double dt_max{0.0};
    double tol_step{0.0};
    int max_steps{0};
    int max_rejects{20};
    double safety{0.8};
    double grow{1.5};
    double shrink{0.5};
    bool adapt_m{false};
    int m_max{0};
    int m_step{0};
};

// Owns one device's matrix, basis and work buffers (through mexk_context_t).
struct DeviceContext {
    int device_id;
    mexk_context_t handle;
    int local_rows;
    int local_nnz;
    int allocated_m_max;

    explicit DeviceContext(int dev_id)
        : device_id(dev_id), handle(nullptr), local_rows(0), local_nnz(0), allocated_m_max(0) {}

    void init_handles();    // selects the device (no library handles exist)
    void create_streams();  // creates the context and its stream
    void alloc_from(const CSRHost& part, int global_cols, int m_alloc_max);
    // The SpMV row-block schedule is built in alloc_from; kept for call-order compatibility.
    void create_descriptors(const CSRHost& part, int global_cols, const CSRHost::GhostMap& ghost_map,
                            int global_row_offset, int m_arnoldi);
    void destroy();
};

struct ArnoldiRunner {
    int num_gpus;
    std::vector<DeviceContext> device_contexts;
    ArnoldiParams params;
    ExpmvMode mode{ExpmvMode::AdaptiveTimeStepping};
    TimeSteppingParams ts_params;
    bool converged = false;
    int restarts_done = 0;
    double last_residual = 0.0;
    std::vector<CSRHost::GhostMap> ghost_maps;

    int global_rows;
    int global_cols;
    long long global_nnz;

    // Extensions (defaults reproduce the reference): arithmetic form, step
    // controller, whether compute_expmv prints the [STEP]/[FLOPs]/METRIC
    // lines, and the statistics of the last solve.
    int precision = MEXK_PREC_FP64;
    int controller = MEXK_CTRL_REFERENCE;
    // 0: orthogonalise against the whole basis; W >= 2: against the last W
    // vectors (mixed precision, symmetric A only; no reference counterpart).
    int ortho_window = 0;
    bool net_loaded = false;
    bool verbose = true;
    // Also print the reference's per-step "H_m column j stored" lines
    // (store_H_column, main.cu:1944-1952) before each attempt's [STEP] line.
    bool log_h_columns = false;
    mexk_result_t last_result{};
    std::vector<mexk_step_t> last_steps;

    ArnoldiRunner(int n_gpus, const ArnoldiParams& arnoldi_params, int total_rows, int total_cols,
                  long long total_nnz);

    void init_all_devices(const std::vector<CSRHost>& partitions, const std::vector<int>& device_ids,
                          const std::vector<CSRHost::GhostMap>& ghost_maps_in);
    // Extension: adopt a context that already holds A (mexk_context_load_bincsr
    // with m_alloc >= params.m); the same checks and messages as init_all_devices.
    void init_from_context(mexk_context_t ctx, int device_id = 0);
    // y_host must hold total_rows entries (the reference writes without resizing).
    void compute_expmv(const std::vector<double>& v_host, std::vector<double>& y_host);
    void destroy();
};
