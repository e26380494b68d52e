// CSRHost: MatrixMarket and Binary CSR v1 loaders, row partitioning and
// ghost maps, with the reference's validation rules, messages and exit
// behaviour (kol-di/matrix-exp-krylov main.cu:86-744, format in
// docs/binary_csr_v1.md).
//
// Loading differs from the reference only in how it reads: Binary CSR
// payloads are read straight into the 32-bit arrays (u32 files) instead of
// being widened to 64-bit copies first, and `.mtx.gz` files are decompressed
// in-process when zlib is available (the reference opens them as plain text,
// main.cu:98).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <limits>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#ifdef MEXK_HAVE_ZLIB
#include <zlib.h>
#endif

#include "matrix_exp_krylov.hpp"

namespace {

[[noreturn]] void fail(const std::string& msg) {
    std::cerr << msg << std::endl;
    std::exit(EXIT_FAILURE);
}

uint32_t le32(const unsigned char* p) {
    return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}
uint64_t le64(const unsigned char* p) { return uint64_t(le32(p)) | (uint64_t(le32(p + 4)) << 32); }

bool ends_with(const std::string& s, const std::string& suf) {
    return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

std::string lower(std::string s) {
    for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    return s;
}

// Reads the whole file as text (gunzipping .gz when built with zlib).
bool read_text(const std::string& path, std::string& out) {
#ifdef MEXK_HAVE_ZLIB
    if (ends_with(path, ".gz")) {
        gzFile gz = gzopen(path.c_str(), "rb");
        if (!gz) return false;
        char buf[1 << 16];
        int got;
        while ((got = gzread(gz, buf, sizeof(buf))) > 0) out.append(buf, static_cast<size_t>(got));
        gzclose(gz);
        return got >= 0;
    }
#endif
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

// Sorted (row, col, value) triples -> CSR with duplicates summed in order.
void assemble(CSRHost& A, std::vector<std::tuple<int, int, double>>& entries) {
    std::sort(entries.begin(), entries.end());
    A.row_ptr.assign(static_cast<size_t>(A.rows) + 1, 0);
    A.col_idx.clear();
    A.values.clear();
    A.col_idx.reserve(entries.size());
    A.values.reserve(entries.size());
    int last_r = -1, last_c = -1;
    for (const auto& e : entries) {
        const int r = std::get<0>(e), c = std::get<1>(e);
        if (r == last_r && c == last_c) {
            A.values.back() += std::get<2>(e);
            continue;
        }
        A.col_idx.push_back(c);
        A.values.push_back(std::get<2>(e));
        A.row_ptr[static_cast<size_t>(r) + 1]++;
        last_r = r;
        last_c = c;
    }
    for (int r = 0; r < A.rows; ++r) A.row_ptr[r + 1] += A.row_ptr[r];
    A.nnz = static_cast<long long>(A.values.size());
}

}  // namespace

void CSRHost::from_matrix_market(const std::string& filename) {
    std::string text;
    if (!read_text(filename, text)) fail("Error: Could not open file " + filename);
    std::istringstream file(text);
    std::string line;
    bool header = false;
    std::string object, format, field, symmetry;
    while (std::getline(file, line)) {
        if (line.empty()) continue;
        std::istringstream ss(line);
        std::string first;
        ss >> first;
        if (lower(first) != "%%matrixmarket") continue;
        ss >> object >> format >> field >> symmetry;
        object = lower(object);
        format = lower(format);
        field = lower(field);
        symmetry = lower(symmetry);
        if (object != "matrix") fail("Error: MatrixMarket object must be 'matrix'");
        if (format != "coordinate") fail("Error: Only 'coordinate' format is supported");
        if (field != "real" && field != "pattern") fail("Error: Only 'real' or 'pattern' fields are supported");
        if (symmetry != "general" && symmetry != "symmetric")
            fail("Error: Only 'general' or 'symmetric' symmetry types are supported");
        header = true;
        break;
    }
    if (!header) fail("Error: Failed to parse MatrixMarket header");
    const bool pattern = field == "pattern";
    const bool symmetric = symmetry == "symmetric";

    bool dims = false;
    while (std::getline(file, line)) {
        if (line.empty() || line[0] == '%') continue;
        std::istringstream ss(line);
        if (!(ss >> rows >> cols >> nnz)) fail("Error: Failed to read matrix dimensions");
        dims = true;
        break;
    }
    if (!dims) fail("Error: Matrix dimensions line not found in file " + filename);

    std::vector<std::tuple<int, int, double>> entries;
    entries.reserve(static_cast<size_t>(nnz) * (symmetric ? 2 : 1));
    long long got = 0;
    while (got < nnz && std::getline(file, line)) {
        if (line.empty() || line[0] == '%') continue;
        std::istringstream ss(line);
        int r, c;
        double v = 1.0;
        if (!(ss >> r >> c)) fail("Error: Failed to read row/col for entry " + std::to_string(got));
        if (!pattern && !(ss >> v)) fail("Error: Failed to read value for entry " + std::to_string(got));
        --r;
        --c;
        if (r < 0 || r >= rows || c < 0 || c >= cols)
            fail("Error: MatrixMarket index out of bounds r=" + std::to_string(r + 1) + " c=" + std::to_string(c + 1));
        entries.emplace_back(r, c, v);
        if (symmetric && r != c) entries.emplace_back(c, r, v);
        ++got;
    }
    if (got != nnz)
        fail("Error: Expected " + std::to_string(nnz) + " entries but read " + std::to_string(got));
    assemble(*this, entries);
}

void CSRHost::from_binary_csr(const std::string& filename) {
    std::ifstream file(filename, std::ios::binary);
    if (!file.is_open()) fail("Error: Could not open binary CSR file " + filename);
    file.seekg(0, std::ios::end);
    const long long file_size = static_cast<long long>(file.tellg());
    file.seekg(0, std::ios::beg);
    if (file_size < 64) fail("Error: Binary CSR file too small (expected at least 64 bytes): " + filename);
    unsigned char h[64];
    file.read(reinterpret_cast<char*>(h), 64);
    if (!file) fail("Error: Failed to read 64-byte header from " + filename);
    static const unsigned char magic[8] = {'C', 'S', 'R', 0, 0, 0, 0, 1};
    if (std::memcmp(h, magic, 8) != 0) fail("Error: Invalid Binary CSR magic in " + filename);
    const uint32_t version = le32(h + 8), flags = le32(h + 12);
    const uint64_t nr = le64(h + 16), nc = le64(h + 24), nz = le64(h + 32);
    const uint32_t idt = le32(h + 40), vdt = le32(h + 44);
    const uint64_t res0 = le64(h + 48), res1 = le64(h + 56);
    if (version != 1) fail("Error: Unsupported Binary CSR version " + std::to_string(version) + " in " + filename);
    if (idt != 1 && idt != 2) fail("Error: Unsupported index_dtype=" + std::to_string(idt) + " in " + filename);
    if (vdt != 1 && vdt != 2) fail("Error: Unsupported value_dtype=" + std::to_string(vdt) + " in " + filename);
    if (res0 != 0 || res1 != 0) fail("Error: Reserved header fields must be zero in " + filename);
    const uint64_t imax = static_cast<uint64_t>(std::numeric_limits<int>::max());
    if (nr > imax || nc > imax || nz > imax)
        fail("Error: Matrix dimensions/nnz exceed int32 limits used by solver in " + filename);
    const uint64_t ib = idt == 1 ? 4 : 8, vb = vdt == 1 ? 4 : 8;
    const uint64_t expected = 64 + (nr + 1) * ib + nz * ib + nz * vb;
    if (expected != static_cast<uint64_t>(file_size))
        fail("Error: Binary CSR size mismatch in " + filename + " (expected " + std::to_string(expected) +
             " bytes, got " + std::to_string(file_size) + ")");

    // Index arrays are kept 64-bit only for u64 files.
    std::vector<uint64_t> ip64, ix64;
    std::vector<uint32_t> ip32, ix32;
    if (idt == 1) {
        ip32.resize(nr + 1);
        ix32.resize(nz);
        file.read(reinterpret_cast<char*>(ip32.data()), static_cast<std::streamsize>(ip32.size() * 4));
        if (!file) fail("Error: Failed to read indptr(u32) from " + filename);
        file.read(reinterpret_cast<char*>(ix32.data()), static_cast<std::streamsize>(ix32.size() * 4));
        if (!file) fail("Error: Failed to read indices(u32) from " + filename);
    } else {
        ip64.resize(nr + 1);
        ix64.resize(nz);
        file.read(reinterpret_cast<char*>(ip64.data()), static_cast<std::streamsize>(ip64.size() * 8));
        if (!file) fail("Error: Failed to read indptr(u64) from " + filename);
        file.read(reinterpret_cast<char*>(ix64.data()), static_cast<std::streamsize>(ix64.size() * 8));
        if (!file) fail("Error: Failed to read indices(u64) from " + filename);
    }
    std::vector<double> data(nz);
    if (vdt == 1) {
        std::vector<float> tmp(nz);
        file.read(reinterpret_cast<char*>(tmp.data()), static_cast<std::streamsize>(tmp.size() * 4));
        if (!file) fail("Error: Failed to read data(f32) from " + filename);
        for (size_t i = 0; i < tmp.size(); ++i) data[i] = static_cast<double>(tmp[i]);
    } else {
        file.read(reinterpret_cast<char*>(data.data()), static_cast<std::streamsize>(data.size() * 8));
        if (!file) fail("Error: Failed to read data(f64) from " + filename);
    }
    auto IP = [&](uint64_t r) -> uint64_t { return idt == 1 ? ip32[r] : ip64[r]; };
    auto IX = [&](uint64_t k) -> uint64_t { return idt == 1 ? ix32[k] : ix64[k]; };

    rows = static_cast<int>(nr);
    cols = static_cast<int>(nc);
    nnz = static_cast<long long>(nz);
    if (IP(0) != 0) fail("Error: indptr[0] must be 0 in " + filename);
    for (uint64_t r = 0; r < nr; ++r)
        if (IP(r) > IP(r + 1))
            fail("Error: indptr is not non-decreasing at row " + std::to_string(r) + " in " + filename);
    if (IP(nr) != nz) fail("Error: indptr[nrows] != nnz in " + filename);
    for (uint64_t k = 0; k < nz; ++k)
        if (IX(k) >= nc) fail("Error: Column index out of range at k=" + std::to_string(k) + " in " + filename);

    const bool sorted = (flags & 1u) != 0, nodup = (flags & 2u) != 0, symu = (flags & 4u) != 0;
    {
        std::ostringstream os;
        os << "Binary CSR header: version=" << version << " flags=0x" << std::hex << flags << std::dec
           << " index_dtype=" << (idt == 1 ? "u32" : "u64") << " value_dtype=" << (vdt == 1 ? "f32" : "f64")
           << " symmetric_upper=" << (symu ? "yes" : "no");
        std::cout << os.str() << std::endl;
    }
    if (sorted || nodup) {
        for (uint64_t r = 0; r < nr; ++r)
            for (uint64_t p = IP(r) + 1; p < IP(r + 1); ++p) {
                if (sorted && IX(p - 1) > IX(p))
                    fail("Error: Row " + std::to_string(r) + " is not sorted but sorted flag is set in " + filename);
                if (nodup && IX(p - 1) == IX(p))
                    fail("Error: Row " + std::to_string(r) + " has duplicates but no_duplicates flag is set in " +
                         filename);
            }
    }
    if (symu) {
        if (rows != cols) fail("Error: symmetric_upper requires square matrix in " + filename);
        std::vector<std::tuple<int, int, double>> entries;
        entries.reserve(static_cast<size_t>(nz) * 2);
        for (uint64_t r = 0; r < nr; ++r)
            for (uint64_t p = IP(r); p < IP(r + 1); ++p) {
                const int c = static_cast<int>(IX(p));
                entries.emplace_back(static_cast<int>(r), c, data[p]);
                if (c != static_cast<int>(r)) entries.emplace_back(c, static_cast<int>(r), data[p]);
            }
        assemble(*this, entries);
        return;
    }
    row_ptr.resize(nr + 1);
    col_idx.resize(nz);
    for (uint64_t r = 0; r <= nr; ++r) row_ptr[r] = static_cast<int>(IP(r));
    for (uint64_t k = 0; k < nz; ++k) col_idx[k] = static_cast<int>(IX(k));
    values.swap(data);
}

std::vector<CSRHost> CSRHost::partition_rows(int num_gpus) const {
    std::vector<CSRHost> parts(static_cast<size_t>(num_gpus));
    const int base = rows / num_gpus, extra = rows % num_gpus;
    int r0 = 0;
    for (int i = 0; i < num_gpus; ++i) {
        const int cnt = base + (i < extra ? 1 : 0);
        CSRHost& P = parts[i];
        P.rows = cnt;
        P.cols = cols;
        if (cnt == 0) {
            P.nnz = 0;
            P.row_ptr.assign(1, 0);
            continue;
        }
        const int e0 = row_ptr[r0], e1 = row_ptr[r0 + cnt];
        P.nnz = e1 - e0;
        P.row_ptr.resize(static_cast<size_t>(cnt) + 1);
        for (int k = 0; k <= cnt; ++k) P.row_ptr[k] = row_ptr[r0 + k] - e0;
        P.col_idx.assign(col_idx.begin() + e0, col_idx.begin() + e1);
        P.values.assign(values.begin() + e0, values.begin() + e1);
        r0 += cnt;
    }
    return parts;
}

CSRHost::GhostMap CSRHost::build_owner_ghost_maps(const std::vector<CSRHost>& parts, int me, int P) const {
    GhostMap g;
    g.send_offsets.assign(P, 0);
    g.send_counts.assign(P, 0);
    g.recv_offsets.assign(P, 0);
    g.recv_counts.assign(P, 0);
    std::vector<int> first(P + 1, 0);
    for (int i = 0; i < P; ++i) first[i + 1] = first[i] + parts[i].rows;
    auto owner_of = [&](int col) {
        return static_cast<int>(std::upper_bound(first.begin(), first.end(), col) - first.begin()) - 1;
    };
    // RECEIVE: columns my rows reference that other partitions own.
    for (long long k = 0; k < parts[me].nnz; ++k) {
        const int col = parts[me].col_idx[k];
        const int o = owner_of(col);
        if (o != me && o >= 0 && o < P) g.owner_to_consumer_map[o].push_back(col);
    }
    size_t off = 0;
    for (int p = 0; p < P; ++p) {
        if (p == me) continue;
        auto& lst = g.owner_to_consumer_map[p];
        std::sort(lst.begin(), lst.end());
        lst.erase(std::unique(lst.begin(), lst.end()), lst.end());
        if (!lst.empty()) {
            g.incoming_peer_info[p] = {off, lst.size()};
            g.recv_offsets[p] = static_cast<int>(off);
            g.recv_counts[p] = static_cast<int>(lst.size());
            g.incoming_global_col_indices.insert(g.incoming_global_col_indices.end(), lst.begin(), lst.end());
            off += lst.size();
        }
    }
    g.total_recv_size = off;
    // SEND: columns I own that other partitions reference.
    for (int p = 0; p < P; ++p) {
        if (p == me) continue;
        auto& lst = g.consumer_to_owner_map[p];
        for (long long k = 0; k < parts[p].nnz; ++k) {
            const int col = parts[p].col_idx[k];
            if (owner_of(col) == me) lst.push_back(col);
        }
        std::sort(lst.begin(), lst.end());
        lst.erase(std::unique(lst.begin(), lst.end()), lst.end());
    }
    off = 0;
    for (int p = 0; p < P; ++p) {
        if (p == me) continue;
        auto& lst = g.consumer_to_owner_map[p];
        if (!lst.empty()) {
            g.outgoing_peer_info[p] = {off, lst.size()};
            g.send_offsets[p] = static_cast<int>(off);
            g.send_counts[p] = static_cast<int>(lst.size());
            g.outgoing_global_col_indices.insert(g.outgoing_global_col_indices.end(), lst.begin(), lst.end());
            off += lst.size();
        }
    }
    g.total_send_size = off;
    return g;
}

void validate_ghost_maps(const std::vector<CSRHost::GhostMap>& maps, int P) {
    auto norm = [](std::vector<int> v) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        return v;
    };
    for (int o = 0; o < P; ++o)
        for (int c = 0; c < P; ++c) {
            if (o == c) continue;
            std::vector<int> send, recv;
            auto s = maps[o].consumer_to_owner_map.find(c);
            if (s != maps[o].consumer_to_owner_map.end()) send = norm(s->second);
            auto r = maps[c].owner_to_consumer_map.find(o);
            if (r != maps[c].owner_to_consumer_map.end()) recv = norm(r->second);
            if (send != recv) {
                std::cerr << "[ERROR] Ghost map mismatch between owner " << o << " and consumer " << c << std::endl;
                std::cerr << "  send size: " << send.size() << " recv size: " << recv.size() << std::endl;
                std::exit(EXIT_FAILURE);
            }
        }
}
