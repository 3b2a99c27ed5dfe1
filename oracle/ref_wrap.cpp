/*
 * ORACLE -- test infrastructure only.
 *
 * extern "C" wrappers around the reference's own CPU kinematics, compiled from
 * the reference's unmodified sources by oracle/Makefile (target "ref") into
 * oracle/_ref/libtplref.so.  Each wrapper follows the reference's torch-facing
 * interface for the same call, minus torch:
 *   ref_a2b_forward / ref_a2b_backward  <- Layers/ReducedModel/Angles2Backbone/angles2backbone_interface.cpp:60-111
 *   ref_a2c_forward / ref_a2c_backward  <- Layers/FullAtomModel/Angles2Coords/angles2coords_interface.cpp:8-115
 *   ref_a2c_save                        <- angles2coords_interface.cpp:117-137 (cConformation::save)
 * The batch is split one chain per call (the reference's batch loops are
 * independent per chain) so that the chains can run on all host threads; the
 * Angles2Coords interface already uses OpenMP over chains
 * (angles2coords_interface.cpp:27,92).
 */
#include <cctype>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cBackboneProteinCPUKernels.hpp"
#include "cConformation.h"
#include "cPDBLoader.h"
#include "nUtil.h"

std::string StringUtil::string_format(const std::string fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt.c_str(), ap);
    va_end(ap);
    return std::string(buf);
}

std::string ProtUtil::convertRes1to3(char r) {
    static const char *one = "GASCVILTRKDNEQMHPFYW";
    static const char *three[] = {"GLY", "ALA", "SER", "CYS", "VAL", "ILE", "LEU", "THR", "ARG", "LYS",
                                  "ASP", "ASN", "GLU", "GLN", "MET", "HIS", "PRO", "PHE", "TYR", "TRP"};
    const char *p = std::strchr(one, r);
    if (!p || !r) throw std::string("Unknown residue name");
    return std::string(three[p - one]);
}

// Math/nUtil.cpp:119-123: whitespace stripped from both ends.
std::string StringUtil::trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

// Math/nUtil.cpp:166-171: C, N, O or S as the first character.
bool ProtUtil::isHeavyAtom(std::string &atom_name) {
    const char c = atom_name.empty() ? '\0' : atom_name[0];
    return c == 'C' || c == 'N' || c == 'O' || c == 'S';
}

extern "C" {

int ref_a2b_forward(double *angles, int *lengths, double *coords, double *A, int B, int L, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int b = 0; b < B; b++)
        cpu_computeCoordinatesBackbone<double>(angles + (size_t)3 * b * L, coords + (size_t)9 * b * L,
                                               A + (size_t)48 * b * L, lengths + b, 1, L);
    return 0;
}

/* dr_dangle is per-chain scratch of 27*L*L doubles for each of `threads` workers. */
int ref_a2b_backward(double *grad_in, double *grad_out, double *angles, int *lengths, double *A,
                     double *dr_dangle, int B, int L, int threads) {
    const size_t per = (size_t)27 * L * L;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int b = 0; b < B; b++) {
        int tid = 0;
#ifdef _OPENMP
        extern int omp_get_thread_num(void);
        tid = omp_get_thread_num();
#endif
        double *dr = dr_dangle + per * tid;
        std::memset(dr, 0, per * sizeof(double));
        cpu_computeDerivativesBackbone<double>(angles + (size_t)3 * b * L, dr, A + (size_t)48 * b * L,
                                               lengths + b, 1, L);
        cpu_backwardFromCoordsBackbone<double>(grad_in + (size_t)3 * b * L, grad_out + (size_t)9 * b * L, dr,
                                               lengths + b, 1, L);
    }
    return 0;
}

int ref_a2c_forward(const unsigned char *seqs, int seq_stride, double *angles, double *coords,
                    unsigned char *res_names, unsigned char *atom_names, int B, int L, int maxA, int threads) {
    int err = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int b = 0; b < B; b++) {
        std::string seq((const char *)seqs + (size_t)b * seq_stride,
                        strnlen((const char *)seqs + (size_t)b * seq_stride, seq_stride));
        std::vector<double> dummy_grad((size_t)8 * L, 0.0);
        try {
            cConformation<double> conf(seq, angles + (size_t)8 * b * L, dummy_grad.data(), L,
                                       coords + (size_t)3 * b * maxA);
            for (size_t j = 0; j < conf.groups.size(); j++)
                for (size_t k = 0; k < conf.groups[j]->atomNames.size(); k++) {
                    int idx = conf.groups[j]->atomIndexes[k];
                    std::string rn = ProtUtil::convertRes1to3(conf.groups[j]->residueName);
                    const std::string &an = conf.groups[j]->atomNames[k];
                    std::memcpy(res_names + ((size_t)b * maxA + idx) * 4, rn.c_str(), rn.size() + 1);
                    std::memcpy(atom_names + ((size_t)b * maxA + idx) * 4, an.c_str(), an.size() + 1);
                }
        } catch (...) {
            err = -3;
        }
    }
    return err;
}

int ref_a2c_backward(double *grad_atoms, double *grad_angles, const unsigned char *seqs, int seq_stride,
                     double *angles, int B, int L, int maxA, int threads) {
    int err = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int b = 0; b < B; b++) {
        std::string seq((const char *)seqs + (size_t)b * seq_stride,
                        strnlen((const char *)seqs + (size_t)b * seq_stride, seq_stride));
        std::vector<double> dummy_coords((size_t)3 * (maxA > 0 ? maxA : 1), 0.0);
        try {
            cConformation<double> conf(seq, angles + (size_t)8 * b * L, grad_angles + (size_t)8 * b * L, L,
                                       dummy_coords.data());
            conf.backward(conf.root, grad_atoms + (size_t)3 * b * maxA);
        } catch (...) {
            err = -3;
        }
    }
    return err;
}

// Angles2Coords_save of one chain: angles [8, len(seq)] (the reference passes the
// sequence length as the row stride), mode 'w' or 'a'.  Returns 0, or -3 if the
// reference threw.
int ref_a2c_save(const char *sequence, double *angles, const char *filename, char mode) {
    std::string seq(sequence);
    std::vector<double> dummy_grad((size_t)8 * seq.size(), 0.0);
    try {
        std::vector<double> coords((size_t)3 * 16 * (seq.size() + 1), 0.0);
        cConformation<double> conf(seq, angles, dummy_grad.data(), (unsigned)seq.size(), coords.data());
        conf.save(std::string(filename), mode);
    } catch (...) {
        return -3;
    }
    return 0;
}

// The reference's PDB reader (cPDBLoader, as PDB2CoordsUnordered uses it): fills up
// to max_atoms atoms (coords xyz, names as NUL-padded 4-byte slots, residue
// numbers) and returns the file's heavy-atom count, or -1 if it cannot be read.
int ref_pdb_read(const char *filename, int max_atoms, double *coords, char *chain_names, char *res_names,
                 int *res_nums, char *atom_names) {
    try {
        cPDBLoader pdb{std::string(filename)};
        const int n = (int)pdb.r.size();
        for (int j = 0; j < n && j < max_atoms; j++) {
            for (int k = 0; k < 3; k++) coords[3 * j + k] = pdb.r[j].v[k];
            std::strncpy(chain_names + 4 * j, pdb.chain_names[j].c_str(), 4);
            std::strncpy(res_names + 4 * j, pdb.res_names[j].c_str(), 4);
            std::strncpy(atom_names + 4 * j, pdb.atom_names[j].c_str(), 4);
            res_nums[j] = pdb.res_nums[j];
        }
        return n;
    } catch (...) {
        return -1;
    }
}
}  // extern "C"
