// Row partitions and ghost maps of the drop-in C++ API (CSRHost::
// partition_rows, build_owner_ghost_maps and validate_ghost_maps, the
// reference's main.cu:526-744), printed for the CPU tests to compare with
// the rules those functions implement. No device work.
//
//   ghost_check matrix.bincsr P [corrupt]
// prints, per partition i:
//   PART i rows nnz
//   RECV i owner col col ...        (owner_to_consumer_map, flattened order)
//   SEND i consumer col col ...     (consumer_to_owner_map)
//   OFFS i total_recv total_send recv_offsets... | send_offsets...
// then validates the maps ("corrupt" drops one entry of the first non-empty
// send list first, which validate_ghost_maps must reject).
#include <cstring>
#include <iostream>
#include <vector>

#include "matrix_exp_krylov.hpp"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: ghost_check matrix.bincsr P [corrupt]" << std::endl;
        return 2;
    }
    CSRHost A;
    A.from_binary_csr(argv[1]);
    const int P = std::atoi(argv[2]);
    std::vector<CSRHost> parts = A.partition_rows(P);
    std::vector<CSRHost::GhostMap> maps;
    for (int i = 0; i < P; ++i) maps.push_back(A.build_owner_ghost_maps(parts, i, P));
    for (int i = 0; i < P; ++i) {
        std::cout << "PART " << i << " " << parts[i].rows << " " << parts[i].nnz << "\n";
        for (const auto& kv : maps[i].owner_to_consumer_map) {
            if (kv.second.empty()) continue;
            std::cout << "RECV " << i << " " << kv.first;
            for (int c : kv.second) std::cout << " " << c;
            std::cout << "\n";
        }
        for (const auto& kv : maps[i].consumer_to_owner_map) {
            if (kv.second.empty()) continue;
            std::cout << "SEND " << i << " " << kv.first;
            for (int c : kv.second) std::cout << " " << c;
            std::cout << "\n";
        }
        std::cout << "OFFS " << i << " " << maps[i].total_recv_size << " " << maps[i].total_send_size;
        for (int o : maps[i].recv_offsets) std::cout << " " << o;
        std::cout << " |";
        for (int o : maps[i].send_offsets) std::cout << " " << o;
        std::cout << "\n";
    }
    std::cout.flush();
    if (argc > 3 && std::strcmp(argv[3], "corrupt") == 0) {
        for (auto& g : maps) {
            bool done = false;
            for (auto& kv : g.consumer_to_owner_map)
                if (!kv.second.empty()) {
                    kv.second.pop_back();
                    done = true;
                    break;
                }
            if (done) break;
        }
    }
    validate_ghost_maps(maps, P);
    std::cout << "VALID" << std::endl;
    return 0;
}
