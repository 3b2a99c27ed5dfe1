// Full-atom residue topology (host and device).
//
// Each residue is a small kinematic tree hanging off the backbone
// (Layers/FullAtomModel/cConformationAA.cpp:3-546 builds it node by node):
//   N joint   (alpha = omega of the previous residue, beta = CA_C_N, d = R_C_N;
//              identity for residue 0)                         atom N
//   CA joint  (alpha = phi)                                     atom CA
//              [Pro: CB, CG, CD fixed in the CA frame, cRigidGroup.cpp:165-172]
//   dummy     (alpha = N_C_CA_CB dihedral constant, beta = 0, d = 0), child of CA,
//             only for residues with a side chain
//   side-chain joints, a linear path below the dummy (chi1..chi5 or a fixed
//             alpha of 0 for Ala's CB), each carrying a rigid group of atoms
//   C joint   (alpha = psi), child of CA                        atoms C, O
//   next residue's N joint is a child of C.
// Output atom order inside a residue: N, CA, side chain (group order), C, O, the
// order of Math/nUtil.cpp:192-517 (getAtomIndex).  Geometry constants follow
// Layers/FullAtomModel/cGeometry.cpp:9-86; local atom positions follow
// Layers/FullAtomModel/cRigidGroup.cpp:30-210.  The carbonyl O sits at bond
// length R_CB_OG (1.417), as in cRigidGroup.cpp:39.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define TPL_HD __host__ __device__
#else
#define TPL_HD
#endif

namespace tpl {

constexpr int kResTypes = 20;
constexpr int kMaxScJoints = 5;
constexpr int kMaxScAtoms = 10;
constexpr int kMaxResAtoms = 14;
// Residue letters in type order.
constexpr char kResLetters[kResTypes + 1] = "GASCVILTRKDNEQMHPFYW";

TPL_HD constexpr int residue_type(unsigned char c) {
    switch (c) {
        case 'G': return 0;  case 'A': return 1;  case 'S': return 2;  case 'C': return 3;
        case 'V': return 4;  case 'I': return 5;  case 'L': return 6;  case 'T': return 7;
        case 'R': return 8;  case 'K': return 9;  case 'D': return 10; case 'N': return 11;
        case 'E': return 12; case 'Q': return 13; case 'M': return 14; case 'H': return 15;
        case 'P': return 16; case 'F': return 17; case 'Y': return 18; case 'W': return 19;
    }
    return -1;
}

TPL_HD constexpr uint32_t pack_name(char a, char b = 0, char c = 0) {
    return (uint32_t)(unsigned char)a | ((uint32_t)(unsigned char)b << 8) | ((uint32_t)(unsigned char)c << 16);
}

template <typename T>
struct Topology {
    // per residue type
    int natoms[kResTypes];
    int njoints[kResTypes];
    int pro[kResTypes];
    uint32_t res_name[kResTypes];
    uint32_t atom_name[kResTypes][kMaxResAtoms];
    // side-chain joints: beta as (cos, sin), bond length, chi row (0..4, -1 = alpha fixed at 0),
    // atom count and first side-chain atom index of the joint's group
    T jcb[kResTypes][kMaxScJoints], jsb[kResTypes][kMaxScJoints], jd[kResTypes][kMaxScJoints];
    int jchi[kResTypes][kMaxScJoints], jna[kResTypes][kMaxScJoints], jfirst[kResTypes][kMaxScJoints];
    T sc[kResTypes][kMaxScAtoms][3];  // side-chain atom positions in their joint's frame
    // shared geometry
    T bb_cb[3], bb_sb[3], bb_d[3];    // backbone joints phi, psi, omega
    T dummy_c, dummy_s;               // Rx of the N-C-CA-CB dihedral constant
    T o_local[3];                     // carbonyl O in the C frame
    T pro_local[3][3];                // Pro CB, CG, CD in the CA frame
    // side-chain atoms past the first of their group (the first sits at the joint's
    // origin), and the groups that carry such atoms, per residue type
    int nextra[kResTypes], nframes[kResTypes];
};

struct TopologyBuilder {
    // Geometry, cGeometry.cpp:9-86 (pi as M_PI there)
    static constexpr double PI = 3.14159265358979323846;
    static constexpr double C_N_CA = PI - 1.9391, N_CA_C = PI - 2.061, CA_C_N = PI - 2.1186, CA_C_O = PI - 2.1033;
    static constexpr double R_CA_C = 1.525, R_C_N = 1.330, R_N_CA = 1.460;
    static constexpr double R_CA_CB = 1.52, C_CA_CB = -(PI - PI * 109.5 / 180.0);
    static constexpr double N_C_CA_CB = 0.5 * PI * 122.6860 / 180.0;
    static constexpr double R_CB_OG = 1.417, CA_CB_OG = PI * 110.773 / 180.0;
    static constexpr double R_CB_SG = 1.808, CA_CB_SG = PI * 113.8169 / 180.0;
    static constexpr double R_CB_CG = 1.527, CA_CB_CG1 = PI * 110.7 / 180.0, CG1_CB_CG2 = 1.88444687881;
    static constexpr double R_CG1_CD1 = 1.52, CB_CG1_CD1 = PI * 113.97 / 180.0;
    static constexpr double CA_CB_OG1 = PI * 109.18 / 180.0, OG1_CB_CG2 = 1.90291866134;
    static constexpr double R_C_C = R_CA_CB, C_C_C = C_CA_CB;
    static constexpr double R_CD_NE = 1.46, R_NE_CZ = 1.33, R_CZ_NH = 1.33;
    static constexpr double CG_CD_NE = -(PI - PI * 111.68 / 180.0), CD_NE_CZ = -(PI - PI * 124.79 / 180.0);
    static constexpr double NE_CZ_NH = PI * 124.79 / 180.0;
    static constexpr double R_CD_CE = 1.46, R_CE_NZ = 1.33, CD_CE_NZ = -(PI - PI * 124.79 / 180.0);
    static constexpr double R_CG_OD = 1.25, CB_CG_OD = PI * 119.22 / 180.0;
    static constexpr double R_CG_OD1 = 1.23, R_CG_ND2 = 1.33, CB_CG_OD1 = PI * 120.85 / 180.0,
                            CB_CG_ND2 = PI * 116.48 / 180.0;
    static constexpr double R_CG_SD = 1.81, R_SD_CE = 1.79, CB_CG_SD = -(PI - PI * 112.69 / 180.0),
                            CG_SD_CE = -(PI - PI * 100.61 / 180.0);
    static constexpr double R_CG_CD2 = 1.35, R_CG_ND1 = 1.38, R_CG_NE2 = 2.1912, R_CG_CE1 = 2.1915;
    static constexpr double CB_CG_CD2 = -(PI - 2.27957453603), CB_CG_ND1 = PI - 2.14413698608,
                            CB_CG_NE2 = -(PI - 2.90352974362), CB_CG_CE1 = PI - 2.75209584734;
};

// Compile-time FP64 cos/sin for the constant tables below (never used at run
// time): reduce x by the nearest multiple of pi/2 (pi/2 split in two doubles,
// Cody-Waite style), then evaluate the Taylor series of sin and cos on
// |r| <= pi/4, where 12 terms are below 1e-20.
struct ConstTrig {
    static constexpr double kHalfPiHi = 1.5707963267948966;
    static constexpr double kHalfPiLo = 6.123233995736766e-17;
    static constexpr void reduce(double x, double &r, int &q) {
        double k = x / kHalfPiHi;
        long n = (long)(k >= 0 ? k + 0.5 : k - 0.5);
        r = (x - (double)n * kHalfPiHi) - (double)n * kHalfPiLo;
        q = (int)(((n % 4) + 4) % 4);
    }
    static constexpr double sin_r(double r) {
        double t = r, sum = r;
        for (int n = 1; n < 12; n++) {
            if (t > -1e-30 && t < 1e-30) break;  // (constant evaluation rejects subnormals)
            t *= -r * r / ((2.0 * n) * (2.0 * n + 1.0));
            sum += t;
        }
        return sum;
    }
    static constexpr double cos_r(double r) {
        double t = 1.0, sum = 1.0;
        for (int n = 1; n < 12; n++) {
            if (t > -1e-30 && t < 1e-30) break;
            t *= -r * r / ((2.0 * n - 1.0) * (2.0 * n));
            sum += t;
        }
        return sum;
    }
    constexpr double s(double x) const {
        double r = 0.0;
        int q = 0;
        reduce(x, r, q);
        return q == 0 ? sin_r(r) : q == 1 ? cos_r(r) : q == 2 ? -sin_r(r) : -cos_r(r);
    }
    constexpr double c(double x) const {
        double r = 0.0;
        int q = 0;
        reduce(x, r, q);
        return q == 0 ? cos_r(r) : q == 1 ? -sin_r(r) : q == 2 ? -cos_r(r) : sin_r(r);
    }
};

// Breakpoint table of sincos_tab (tpl_common.cuh): (sin, cos)(k pi/32) for
// k = -32..32 as hi + lo float pairs.
struct SinCosTableC {
    float v[65][4];
};
constexpr SinCosTableC make_sincos_table() {
    SinCosTableC t{};
    const ConstTrig trig{};
    for (int i = 0; i <= 64; i++) {
        const double a = (i - 32) * (3.14159265358979323846 / 32.0);
        const double s = trig.s(a), c = trig.c(a);
        const float sh = (float)s, ch = (float)c;
        t.v[i][0] = sh;
        t.v[i][1] = ch;
        t.v[i][2] = (float)(s - (double)sh);
        t.v[i][3] = (float)(c - (double)ch);
    }
    return t;
}

// The topology in precision T, from the FP64 geometry (evaluated at compile time).
template <typename T>
constexpr Topology<T> make_topology() {
    Topology<T> tp{};
    const ConstTrig trig{};
    using G = TopologyBuilder;
    const double h = G::PI / 2.0;
    for (int t = 0; t < kResTypes; t++) {
        tp.njoints[t] = 0;
        tp.pro[t] = 0;
        for (int k = 0; k < kMaxScJoints; k++) {
            tp.jcb[t][k] = T(1); tp.jsb[t][k] = T(0); tp.jd[t][k] = T(0);
            tp.jchi[t][k] = -1; tp.jna[t][k] = 0; tp.jfirst[t][k] = 0;
        }
        for (int a = 0; a < kMaxScAtoms; a++) tp.sc[t][a][0] = tp.sc[t][a][1] = tp.sc[t][a][2] = T(0);
        for (int a = 0; a < kMaxResAtoms; a++) tp.atom_name[t][a] = 0;
    }
    int t = 0, nsc = 0;
    auto res = [&](int type, char a, char b, char c) {
        t = type;
        nsc = 0;
        tp.res_name[t] = pack_name(a, b, c);
    };
    auto joint = [&](int chi, double beta, double d) {
        int k = tp.njoints[t]++;
        tp.jcb[t][k] = T(trig.c(beta));
        tp.jsb[t][k] = T(trig.s(beta));
        tp.jd[t][k] = T(d);
        tp.jchi[t][k] = chi;
        tp.jfirst[t][k] = nsc;
    };
    auto atom = [&](uint32_t name, double x, double y, double z) {
        int k = tp.njoints[t] - 1;
        tp.sc[t][nsc][0] = T(x); tp.sc[t][nsc][1] = T(y); tp.sc[t][nsc][2] = T(z);
        tp.atom_name[t][2 + nsc] = name;
        tp.jna[t][k]++;
        nsc++;
    };
    const double cv = trig.c(G::CA_CB_CG1 - h), sv = trig.s(G::CA_CB_CG1 - h);
    // G
    res(0, 'G', 'L', 'Y');
    // A: CB on a joint with alpha fixed at 0 (cConformationAA.cpp:90)
    res(1, 'A', 'L', 'A'); joint(-1, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    // S
    res(2, 'S', 'E', 'R'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    atom(pack_name('O', 'G'), G::R_CB_OG * trig.c(-(G::PI - G::CA_CB_OG)), 0, G::R_CB_OG * trig.s(-(G::PI - G::CA_CB_OG)));
    // C
    res(3, 'C', 'Y', 'S'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    atom(pack_name('S', 'G'), G::R_CB_SG * trig.c(-(G::PI - G::CA_CB_SG)), 0, G::R_CB_SG * trig.s(-(G::PI - G::CA_CB_SG)));
    // V
    res(4, 'V', 'A', 'L'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    atom(pack_name('C', 'G', '1'), G::R_CB_CG * sv, G::R_CB_CG * cv * trig.s(G::CG1_CB_CG2 / 2), G::R_CB_CG * cv * trig.c(G::CG1_CB_CG2 / 2));
    atom(pack_name('C', 'G', '2'), G::R_CB_CG * sv, -G::R_CB_CG * cv * trig.s(G::CG1_CB_CG2 / 2), G::R_CB_CG * cv * trig.c(G::CG1_CB_CG2 / 2));
    // I: group 1 (CB, CG2) on chi1, group 2 (CG1, CD1) on chi2
    res(5, 'I', 'L', 'E'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    atom(pack_name('C', 'G', '2'), G::R_CB_CG * sv, G::R_CB_CG * cv * trig.s(G::CG1_CB_CG2), G::R_CB_CG * cv * trig.c(G::CG1_CB_CG2));
    joint(1, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'G', '1'), 0, 0, 0);
    atom(pack_name('C', 'D', '1'), G::R_CG1_CD1 * trig.c(G::PI - G::CB_CG1_CD1), 0, -G::R_CG1_CD1 * trig.s(G::PI - G::CB_CG1_CD1));
    // L
    res(6, 'L', 'E', 'U'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('C', 'D', '1'), G::R_CB_CG * sv, G::R_CB_CG * cv * trig.s(G::CG1_CB_CG2 / 2), G::R_CB_CG * cv * trig.c(G::CG1_CB_CG2 / 2));
    atom(pack_name('C', 'D', '2'), G::R_CB_CG * sv, -G::R_CB_CG * cv * trig.s(G::CG1_CB_CG2 / 2), G::R_CB_CG * cv * trig.c(G::CG1_CB_CG2 / 2));
    // T (OG1 uses R_CB_OG, as cRigidGroup.cpp:110)
    res(7, 'T', 'H', 'R'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    {
        const double co = trig.c(G::CA_CB_OG1 - h), so = trig.s(G::CA_CB_OG1 - h);
        atom(pack_name('O', 'G', '1'), G::R_CB_OG * so, G::R_CB_OG * co * trig.s(G::OG1_CB_CG2 / 2), G::R_CB_OG * co * trig.c(G::OG1_CB_CG2 / 2));
        atom(pack_name('C', 'G', '2'), G::R_CB_CG * sv, -G::R_CB_CG * cv * trig.s(G::OG1_CB_CG2 / 2), G::R_CB_CG * cv * trig.c(G::OG1_CB_CG2 / 2));
    }
    // R
    res(8, 'A', 'R', 'G'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    joint(2, G::C_C_C, G::R_C_C); atom(pack_name('C', 'D'), 0, 0, 0);
    joint(3, G::CG_CD_NE, G::R_CD_NE); atom(pack_name('N', 'E'), 0, 0, 0);
    joint(4, G::CD_NE_CZ, G::R_NE_CZ); atom(pack_name('C', 'Z'), 0, 0, 0);
    atom(pack_name('N', 'H', '1'), G::R_CZ_NH * trig.s(G::NE_CZ_NH - h), 0, G::R_CZ_NH * trig.c(G::NE_CZ_NH - h));
    atom(pack_name('N', 'H', '2'), G::R_CZ_NH * trig.s(G::NE_CZ_NH - h), 0, -G::R_CZ_NH * trig.c(G::NE_CZ_NH - h));
    // K
    res(9, 'L', 'Y', 'S'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    joint(2, G::C_C_C, G::R_C_C); atom(pack_name('C', 'D'), 0, 0, 0);
    joint(3, G::C_C_C, G::R_CD_CE); atom(pack_name('C', 'E'), 0, 0, 0);
    joint(4, G::CD_CE_NZ, G::R_CE_NZ); atom(pack_name('N', 'Z'), 0, 0, 0);
    // D
    res(10, 'A', 'S', 'P'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('O', 'D', '1'), G::R_CG_OD * trig.s(G::CB_CG_OD - h), 0, G::R_CG_OD * trig.c(G::CB_CG_OD - h));
    atom(pack_name('O', 'D', '2'), G::R_CG_OD * trig.s(G::CB_CG_OD - h), 0, -G::R_CG_OD * trig.c(G::CB_CG_OD - h));
    // N
    res(11, 'A', 'S', 'N'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('O', 'D', '1'), G::R_CG_OD1 * trig.s(G::CB_CG_OD1 - h), 0, G::R_CG_OD1 * trig.c(G::CB_CG_OD1 - h));
    atom(pack_name('N', 'D', '2'), G::R_CG_ND2 * trig.s(G::CB_CG_ND2 - h), 0, -G::R_CG_ND2 * trig.c(G::CB_CG_ND2 - h));
    // E
    res(12, 'G', 'L', 'U'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    joint(2, G::C_C_C, G::R_C_C); atom(pack_name('C', 'D'), 0, 0, 0);
    atom(pack_name('O', 'E', '1'), G::R_CG_OD * trig.s(G::CB_CG_OD - h), 0, G::R_CG_OD * trig.c(G::CB_CG_OD - h));
    atom(pack_name('O', 'E', '2'), G::R_CG_OD * trig.s(G::CB_CG_OD - h), 0, -G::R_CG_OD * trig.c(G::CB_CG_OD - h));
    // Q
    res(13, 'G', 'L', 'N'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    joint(2, G::C_C_C, G::R_C_C); atom(pack_name('C', 'D'), 0, 0, 0);
    atom(pack_name('O', 'E', '1'), G::R_CG_OD1 * trig.s(G::CB_CG_OD1 - h), 0, G::R_CG_OD1 * trig.c(G::CB_CG_OD1 - h));
    atom(pack_name('N', 'E', '2'), G::R_CG_ND2 * trig.s(G::CB_CG_ND2 - h), 0, -G::R_CG_ND2 * trig.c(G::CB_CG_ND2 - h));
    // M
    res(14, 'M', 'E', 'T'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    joint(2, G::CB_CG_SD, G::R_CG_SD); atom(pack_name('S', 'D'), 0, 0, 0);
    joint(3, G::CG_SD_CE, G::R_SD_CE); atom(pack_name('C', 'E'), 0, 0, 0);
    // H
    res(15, 'H', 'I', 'S'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('C', 'D', '2'), G::R_CG_CD2 * trig.c(G::CB_CG_CD2), G::R_CG_CD2 * trig.s(G::CB_CG_CD2), 0);
    atom(pack_name('N', 'E', '2'), G::R_CG_NE2 * trig.c(G::CB_CG_NE2), G::R_CG_NE2 * trig.s(G::CB_CG_NE2), 0);
    atom(pack_name('C', 'E', '1'), G::R_CG_CE1 * trig.c(G::CB_CG_CE1), G::R_CG_CE1 * trig.s(G::CB_CG_CE1), 0);
    atom(pack_name('N', 'D', '1'), G::R_CG_ND1 * trig.c(G::CB_CG_ND1), G::R_CG_ND1 * trig.s(G::CB_CG_ND1), 0);
    // P: no side-chain joint; CB, CG, CD ride on the CA frame
    res(16, 'P', 'R', 'O'); tp.pro[16] = 1;
    tp.atom_name[16][2] = pack_name('C', 'B'); tp.atom_name[16][3] = pack_name('C', 'G'); tp.atom_name[16][4] = pack_name('C', 'D');
    // F
    res(17, 'P', 'H', 'E'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('C', 'D', '1'), 0.69229424, -1.20533343, 0);
    atom(pack_name('C', 'E', '1'), 2.08228309, -1.20846014, 0);
    atom(pack_name('C', 'Z'), 2.77997771, -0.00625341, 0);
    atom(pack_name('C', 'E', '2'), 2.08768347, 1.19908002, 0);
    atom(pack_name('C', 'D', '2'), 0.69769462, 1.20220673, 0);
    // Y
    res(18, 'T', 'Y', 'R'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('C', 'D', '1'), 0.69229424, -1.20533343, 0);
    atom(pack_name('C', 'E', '1'), 2.08228309, -1.20846014, 0);
    atom(pack_name('C', 'Z'), 2.77997771, -0.00625341, 0);
    atom(pack_name('C', 'E', '2'), 2.08768347, 1.19908002, 0);
    atom(pack_name('C', 'D', '2'), 0.69769462, 1.20220673, 0);
    atom(pack_name('O', 'H'), 4.16960749, 0.05377697, 0);
    // W
    res(19, 'T', 'R', 'P'); joint(0, G::C_CA_CB, G::R_CA_CB); atom(pack_name('C', 'B'), 0, 0, 0);
    joint(1, G::C_C_C, G::R_C_C); atom(pack_name('C', 'G'), 0, 0, 0);
    atom(pack_name('C', 'D', '1'), 0.829890578, -1.09003744, 0);
    atom(pack_name('C', 'D', '2'), 0.84949676, 1.15028973, 0);
    atom(pack_name('N', 'E', '1'), 2.1363699, -0.64570528, 0);
    atom(pack_name('C', 'E', '2'), 2.18136443, 0.71889842, 0);
    atom(pack_name('C', 'E', '3'), 0.61303306, 2.5301684, 0);
    atom(pack_name('C', 'Z', '2'), 3.22086556, 1.65663275, 0);
    atom(pack_name('C', 'Z', '3'), 1.68979906, 3.42486545, 0);
    atom(pack_name('C', 'H', '2'), 2.92849902, 3.0257584, 0);

    // atom counts, backbone names
    for (int r = 0; r < kResTypes; r++) {
        int sc = 0;
        tp.nextra[r] = tp.nframes[r] = 0;
        for (int k = 0; k < tp.njoints[r]; k++) {
            sc += tp.jna[r][k];
            if (tp.jna[r][k] > 1) {
                tp.nextra[r] += tp.jna[r][k] - 1;
                tp.nframes[r]++;
            }
        }
        if (tp.pro[r]) sc = 3;
        tp.natoms[r] = 4 + sc;
        tp.atom_name[r][0] = pack_name('N');
        tp.atom_name[r][1] = pack_name('C', 'A');
        tp.atom_name[r][tp.natoms[r] - 2] = pack_name('C');
        tp.atom_name[r][tp.natoms[r] - 1] = pack_name('O');
    }
    const double bb_beta[3] = {G::C_N_CA, G::N_CA_C, G::CA_C_N};
    const double bb_d[3] = {G::R_N_CA, G::R_CA_C, G::R_C_N};
    for (int k = 0; k < 3; k++) {
        tp.bb_cb[k] = T(trig.c(bb_beta[k]));
        tp.bb_sb[k] = T(trig.s(bb_beta[k]));
        tp.bb_d[k] = T(bb_d[k]);
    }
    tp.dummy_c = T(trig.c(G::N_C_CA_CB));
    tp.dummy_s = T(trig.s(G::N_C_CA_CB));
    tp.o_local[0] = T(G::R_CB_OG * trig.c(G::CA_C_O));
    tp.o_local[1] = T(0);
    tp.o_local[2] = T(G::R_CB_OG * trig.s(G::CA_C_O));
    const double pro[3][3] = {{0.36842372, -1.29540981, 0.70468246},
                              {-0.76137817, -2.21546205, 0.39299099},
                              {-1.97838492, -1.33927458, 0.35849352}};
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++) tp.pro_local[a][c] = T(pro[a][c]);
    return tp;
}

// Facts the chunked Angles2Coords forward relies on: side-chain joint k reads chi
// angle k (or none: alpha fixed at 0, Ala), every group's first atom sits at its
// joint's origin, and at most two groups per residue carry further atoms.
constexpr bool topology_layout_ok() {
    const Topology<double> tp = make_topology<double>();
    for (int t = 0; t < kResTypes; t++) {
        if (tp.nframes[t] > 2) return false;
        for (int k = 0; k < tp.njoints[t]; k++) {
            if (tp.jchi[t][k] != k && tp.jchi[t][k] != -1) return false;
            const int f0 = tp.jfirst[t][k];
            if (tp.jna[t][k] < 1 || tp.sc[t][f0][0] != 0.0 || tp.sc[t][f0][1] != 0.0 || tp.sc[t][f0][2] != 0.0)
                return false;
        }
    }
    return true;
}
static_assert(topology_layout_ok(), "side-chain layout assumed by the chunked forward");

}  // namespace tpl
