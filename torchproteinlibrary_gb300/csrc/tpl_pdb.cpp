// PDB reading on the host (native C++), the on-disk format ahead of the path.
//
// Reads the heavy-atom ATOM records of a PDB file the way cPDBLoader
// (Layers/FullAtomModel/cPDBLoader.cpp:25-55) does for PDB2CoordsUnordered
// (Layers/FullAtomModel/PDB2Coords/pdb2coords_interface.cpp:75-127):
//   * a record is a line whose first four characters are "ATOM" (HETATM is not);
//   * atom name = columns 13-16 without surrounding whitespace; only names that
//     start with C, N, O or S (heavy atoms) are kept;
//   * x, y, z = columns 31-38, 39-46, 47-54, each parsed as a 32-bit float and
//     widened to double (the reference parses with std::stof);
//   * residue name = columns 18-20, chain = column 22 (whitespace-trimmed),
//     residue number = columns 23-26 as an integer;
//   * names go to NUL-padded 4-byte slots.
// Lines too short to hold the fields are skipped (the reference's substr throws
// there).  Files of a batch are read by a pool of host threads.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tpl_gb300.h"

namespace {

struct PdbAtom {
    double x, y, z;
    char chain[4], res[4], atom[4];
    int32_t res_num;
};

std::string trimmed(const std::string &s, size_t pos, size_t len) {
    if (pos >= s.size()) return std::string();
    std::string f = s.substr(pos, len);
    size_t a = 0, b = f.size();
    while (a < b && std::isspace((unsigned char)f[a])) a++;
    while (b > a && std::isspace((unsigned char)f[b - 1])) b--;
    return f.substr(a, b - a);
}

void to_slot(const std::string &s, char *slot) {
    std::memset(slot, 0, 4);
    std::memcpy(slot, s.data(), std::min<size_t>(4, s.size()));
}

bool parse_float(const std::string &line, size_t pos, double *out) {
    if (pos >= line.size()) return false;
    const std::string f = line.substr(pos, 8);
    char *end = nullptr;
    const float v = std::strtof(f.c_str(), &end);
    if (end == f.c_str()) return false;
    *out = (double)v;
    return true;
}

bool parse_int(const std::string &line, size_t pos, int32_t *out) {
    if (pos >= line.size()) return false;
    const std::string f = line.substr(pos, 4);
    char *end = nullptr;
    const long v = std::strtol(f.c_str(), &end, 10);
    if (end == f.c_str()) return false;
    *out = (int32_t)v;
    return true;
}

// Heavy-atom ATOM records of one file; false if the file cannot be opened.
bool read_atoms(const char *filename, std::vector<PdbAtom> &atoms) {
    std::ifstream in(filename);
    if (!in) return false;
    std::string line;
    while (std::getline(in, line)) {
        if (line.compare(0, 4, "ATOM") != 0) continue;
        const std::string name = trimmed(line, 12, 4);
        if (name.empty()) continue;
        const char c = name[0];
        if (!(c == 'C' || c == 'N' || c == 'O' || c == 'S')) continue;
        PdbAtom a{};
        if (!parse_float(line, 30, &a.x) || !parse_float(line, 38, &a.y) || !parse_float(line, 46, &a.z)) continue;
        if (!parse_int(line, 22, &a.res_num)) continue;
        to_slot(trimmed(line, 17, 3), a.res);
        to_slot(trimmed(line, 21, 1), a.chain);
        to_slot(name, a.atom);
        atoms.push_back(a);
    }
    return true;
}

}  // namespace

extern "C" {

int tpl_pdb_count_atoms(const char *filename, int32_t *num_atoms) {
    if (!filename || !num_atoms) return TPL_ERR_ARGUMENT;
    std::vector<PdbAtom> atoms;
    if (!read_atoms(filename, atoms)) return TPL_ERR_IO;
    *num_atoms = (int32_t)atoms.size();
    return TPL_OK;
}

int tpl_pdb_read_batch(const char *const *filenames, int batch, int max_atoms, double *coords, uint8_t *chain_names,
                       uint8_t *res_names, int32_t *res_nums, uint8_t *atom_names, int32_t *num_atoms, int threads) {
    if (batch < 0 || max_atoms < 0) return TPL_ERR_ARGUMENT;
    if (batch == 0) return TPL_OK;
    if (!filenames || !num_atoms || (max_atoms > 0 && (!coords || !chain_names || !res_names || !res_nums ||
                                                       !atom_names)))
        return TPL_ERR_ARGUMENT;
    std::atomic<int> next{0}, status{TPL_OK};
    auto work = [&]() {
        std::vector<PdbAtom> atoms;
        for (int b = next++; b < batch; b = next++) {
            atoms.clear();
            if (!filenames[b] || !read_atoms(filenames[b], atoms)) {
                int expect = TPL_OK;
                status.compare_exchange_strong(expect, TPL_ERR_IO);
                num_atoms[b] = 0;
                continue;
            }
            const int n = (int)atoms.size();
            num_atoms[b] = n;
            if (n > max_atoms) {
                int expect = TPL_OK;
                status.compare_exchange_strong(expect, TPL_ERR_ATOMS);
            }
            const size_t row = (size_t)b * max_atoms;
            std::memset(coords + 3 * row, 0, sizeof(double) * 3 * max_atoms);
            std::memset(chain_names + 4 * row, 0, 4 * (size_t)max_atoms);
            std::memset(res_names + 4 * row, 0, 4 * (size_t)max_atoms);
            std::memset(atom_names + 4 * row, 0, 4 * (size_t)max_atoms);
            std::memset(res_nums + row, 0, sizeof(int32_t) * max_atoms);
            for (int j = 0; j < std::min(n, max_atoms); j++) {
                const PdbAtom &a = atoms[j];
                coords[3 * (row + j)] = a.x;
                coords[3 * (row + j) + 1] = a.y;
                coords[3 * (row + j) + 2] = a.z;
                std::memcpy(chain_names + 4 * (row + j), a.chain, 4);
                std::memcpy(res_names + 4 * (row + j), a.res, 4);
                std::memcpy(atom_names + 4 * (row + j), a.atom, 4);
                res_nums[row + j] = a.res_num;
            }
        }
    };
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    nt = std::max(1, std::min(nt, batch));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    return status.load();
}

}  // extern "C"
