/*
 * ORACLE -- test infrastructure only.
 *
 * Plain-C FP64 restatement of TorchProteinLibrary's CPU algorithms for the
 * internal-coordinate chain kinematics path.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference legs may load this library,
 * and only as the checker or the timed CPU baseline.  The product path never
 * calls it.
 *
 * Pinned against the reference itself: oracle/Makefile builds the reference's
 * own kinematics sources (unmodified) into oracle/_ref/, and
 * tests/test_oracle_pin.py plus tests/golden/make_golden.py compare the two.
 *
 * What is restated (reference paths are relative to the reference project):
 *   - Angles2Backbone forward: Layers/ReducedModel/cBackboneProteinCPUKernels.cpp:14-60
 *     (serial chain product A_i = A_{i-1} B_i, x_i = translation(A_i)).
 *   - Angles2Backbone backward: cBackboneProteinCPUKernels.cpp:62-145 (per (angle, atom)
 *     Jacobian A_{m-1} dB A_m^{-1} A_i applied to the origin, then dL/dangle =
 *     sum_i g_i . dx_i/dangle).  The Jacobian is accumulated on the fly instead
 *     of being materialised as dr_dangle[B,3,27L^2].
 *     Deliberate difference: omega of the last residue reads A[3*len] in the
 *     reference (one past the chain, cBackboneProteinCPUKernels.cpp:83); the
 *     oracle returns 0 there, which is the exact derivative.
 *   - Angles2Coords forward/backward: Layers/FullAtomModel/cConformation.cpp:30-211,
 *     cConformationAA.cpp:3-546, cRigidGroup.cpp:17-210, cGeometry.cpp:9-86,
 *     Angles2Coords/angles2coords_interface.cpp:8-115 (tree of rigid groups, DFS
 *     forward M = M_parent * Ry(beta) Tx(d) Rx(alpha); backward for every joint
 *     with a gradient slot: sum over subtree atoms of g . (M_parent dM M^{-1}) x).
 *   - Atom counts and names: Math/nUtil.cpp:174-565.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.14159265358979323846

/* ---------------------------------------------------------------- 4x4 helpers */
typedef struct { double m[16]; } M44;

static void m44_identity(M44 *a) {
    memset(a->m, 0, sizeof(a->m));
    a->m[0] = a->m[5] = a->m[10] = a->m[15] = 1.0;
}
static M44 m44_mul(const M44 *a, const M44 *b) {
    M44 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0.0;
            for (int k = 0; k < 4; k++) s += a->m[4 * i + k] * b->m[4 * k + j];
            r.m[4 * i + j] = s;
        }
    return r;
}
/* rigid inverse (transpose rotation, -R^T t), Math/cMatrix44.cpp:142-153 */
static M44 m44_rigid_inverse(const M44 *a) {
    M44 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[4 * i + j] = a->m[4 * j + i];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int j = 0; j < 3; j++) s += r.m[4 * i + j] * a->m[4 * j + 3];
        r.m[4 * i + 3] = -s;
    }
    r.m[12] = r.m[13] = r.m[14] = 0.0;
    r.m[15] = 1.0;
    return r;
}
static void m44_apply(const M44 *a, const double *v, double *out) {
    double x = v[0], y = v[1], z = v[2];
    for (int i = 0; i < 3; i++)
        out[i] = a->m[4 * i] * x + a->m[4 * i + 1] * y + a->m[4 * i + 2] * z + a->m[4 * i + 3];
}
/* B(alpha, beta, d) = Ry(beta) Tx(d) Rx(alpha), written out as in Math/cMatrix44.cpp:47-52 */
static void bond_matrix(M44 *b, double alpha, double beta, double d) {
    double ca = cos(alpha), sa = sin(alpha), cb = cos(beta), sb = sin(beta);
    double *m = b->m;
    m[0] = cb;  m[1] = sa * sb; m[2] = ca * sb;  m[3] = d * cb;
    m[4] = 0.0; m[5] = ca;      m[6] = -sa;      m[7] = 0.0;
    m[8] = -sb; m[9] = sa * cb; m[10] = ca * cb; m[11] = -d * sb;
    m[12] = 0.0; m[13] = 0.0; m[14] = 0.0; m[15] = 1.0;
}
/* dB/dalpha, Math/cMatrix44.cpp:54-59 */
static void bond_matrix_dalpha(M44 *b, double alpha, double beta) {
    double ca = cos(alpha), sa = sin(alpha), cb = cos(beta), sb = sin(beta);
    double *m = b->m;
    m[0] = 0.0; m[1] = ca * sb;  m[2] = -sa * sb; m[3] = 0.0;
    m[4] = 0.0; m[5] = -sa;      m[6] = -ca;      m[7] = 0.0;
    m[8] = 0.0; m[9] = ca * cb;  m[10] = -sa * cb; m[11] = 0.0;
    m[12] = m[13] = m[14] = m[15] = 0.0;
}
/* The reference full-atom transforms build the same matrices from three
 * factors (cConformation.cpp:7-20): Ry(beta) * T_x(d) * Rx(alpha). */
static void ry(M44 *r, double a) {
    m44_identity(r);
    r->m[0] = cos(a); r->m[2] = sin(a); r->m[8] = -sin(a); r->m[10] = cos(a);
}
static void rx(M44 *r, double a) {
    m44_identity(r);
    r->m[5] = cos(a); r->m[6] = -sin(a); r->m[9] = sin(a); r->m[10] = cos(a);
}
static void drx(M44 *r, double a) {
    memset(r->m, 0, sizeof(r->m));
    r->m[5] = -sin(a); r->m[6] = -cos(a); r->m[9] = cos(a); r->m[10] = -sin(a);
}
static void tx(M44 *r, double d) { m44_identity(r); r->m[3] = d; }
static void joint_matrices(double alpha, double beta, double d, M44 *mat, M44 *dmat) {
    M44 Ry, T, Rx, dRx, RyT;
    ry(&Ry, beta); tx(&T, d); rx(&Rx, alpha); drx(&dRx, alpha);
    RyT = m44_mul(&Ry, &T);
    *mat = m44_mul(&RyT, &Rx);
    *dmat = m44_mul(&RyT, &dRx);
}

/* ------------------------------------------------- Angles2Backbone constants */
/* cBackboneProteinCPUKernels.cpp:6-12 */
static const double R_CA_C = 1.525, R_C_N = 1.330, R_N_CA = 1.460;
#define BB_CA_C_N (PI - 2.1186)
#define BB_C_N_CA (PI - 1.9391)
#define BB_N_CA_C (PI - 2.061)

int oracle_a2b_forward(const double *angles, const int *lengths, double *coords, double *A,
                       int B, int L) {
    const int atoms_stride = 3 * L;
    for (int b = 0; b < B; b++) {
        int len = lengths[b];
        if (len < 0 || len > L) return -1;
        const double *phi = angles + (size_t)(3 * b) * L;
        const double *psi = angles + (size_t)(3 * b + 1) * L;
        const double *omega = angles + (size_t)(3 * b + 2) * L;
        double *x = coords + (size_t)b * atoms_stride * 3;
        M44 *Ab = (M44 *)(A + (size_t)b * atoms_stride * 16);
        memset(x, 0, sizeof(double) * 3 * atoms_stride);
        memset(Ab, 0, sizeof(M44) * atoms_stride);
        if (len == 0) continue;
        m44_identity(&Ab[0]);
        for (int i = 1; i < 3 * len; i++) {
            int j = i / 3;
            M44 Bm;
            if (i % 3 == 1) bond_matrix(&Bm, phi[j], BB_C_N_CA, R_N_CA);
            else if (i % 3 == 2) bond_matrix(&Bm, psi[j], BB_N_CA_C, R_CA_C);
            else bond_matrix(&Bm, omega[j - 1], BB_CA_C_N, R_C_N);
            Ab[i] = m44_mul(&Ab[i - 1], &Bm);
            x[3 * i + 0] = Ab[i].m[3];
            x[3 * i + 1] = Ab[i].m[7];
            x[3 * i + 2] = Ab[i].m[11];
        }
    }
    return 0;
}

int oracle_a2b_backward(double *grad_angles, const double *grad_coords, const double *angles,
                        const int *lengths, const double *A, int B, int L) {
    const int atoms_stride = 3 * L;
    const double bangle[3] = {BB_C_N_CA, BB_N_CA_C, BB_CA_C_N};
    for (int b = 0; b < B; b++) {
        int len = lengths[b];
        if (len < 0 || len > L) return -1;
        const M44 *Ab = (const M44 *)(A + (size_t)b * atoms_stride * 16);
        const double *g = grad_coords + (size_t)b * atoms_stride * 3;
        for (int k = 0; k < 3; k++) {
            const double *ang = angles + (size_t)(3 * b + k) * L;
            double *out = grad_angles + (size_t)(3 * b + k) * L;
            for (int j = 0; j < L; j++) out[j] = 0.0;
            for (int j = 0; j < len; j++) {
                int m = 3 * j + k + 1; /* the atom whose frame the angle rotates */
                if (m >= 3 * len) continue; /* omega of the last residue moves nothing */
                M44 dB, Ainv, left, F;
                bond_matrix_dalpha(&dB, ang[j], bangle[k]);
                Ainv = m44_rigid_inverse(&Ab[m]);
                left = m44_mul(&Ab[m - 1], &dB);
                F = m44_mul(&left, &Ainv);
                double s = 0.0;
                for (int i = m - 1; i < 3 * len; i++) {
                    M44 Fi = m44_mul(&F, &Ab[i]);
                    s += g[3 * i] * Fi.m[3] + g[3 * i + 1] * Fi.m[7] + g[3 * i + 2] * Fi.m[11];
                }
                out[j] = s;
            }
        }
    }
    return 0;
}

/* --------------------------------------------------- Angles2Coords topology */
/* Geometry, cGeometry.cpp:9-86 */
#define G_C_N_CA (PI - 1.9391)
#define G_N_CA_C (PI - 2.061)
#define G_CA_C_N (PI - 2.1186)
#define G_CA_C_O (PI - 2.1033)
#define G_R_CA_CB 1.52
#define G_C_CA_CB (-(PI - PI * 109.5 / 180.0))
#define G_N_C_CA_CB (0.5 * PI * 122.6860 / 180.0)
#define G_R_CB_OG 1.417
#define G_CA_CB_OG (PI * 110.773 / 180.0)
#define G_R_CB_SG 1.808
#define G_CA_CB_SG (PI * 113.8169 / 180.0)
#define G_R_CB_CG 1.527
#define G_CA_CB_CG1 (PI * 110.7 / 180.0)
#define G_CG1_CB_CG2 1.88444687881
#define G_R_CG1_CD1 1.52
#define G_CB_CG1_CD1 (PI * 113.97 / 180.0)
#define G_CA_CB_OG1 (PI * 109.18 / 180.0)
#define G_OG1_CB_CG2 1.90291866134
#define G_R_C_C G_R_CA_CB
#define G_C_C_C G_C_CA_CB
#define G_R_CD_NE 1.46
#define G_R_NE_CZ 1.33
#define G_R_CZ_NH 1.33
#define G_CG_CD_NE (-(PI - PI * 111.68 / 180.0))
#define G_CD_NE_CZ (-(PI - PI * 124.79 / 180.0))
#define G_NE_CZ_NH (PI * 124.79 / 180.0)
#define G_R_CD_CE 1.46
#define G_R_CE_NZ 1.33
#define G_CD_CE_NZ (-(PI - PI * 124.79 / 180.0))
#define G_R_CG_OD 1.25
#define G_CB_CG_OD (PI * 119.22 / 180.0)
#define G_R_CG_OD1 1.23
#define G_R_CG_ND2 1.33
#define G_CB_CG_OD1 (PI * 120.85 / 180.0)
#define G_CB_CG_ND2 (PI * 116.48 / 180.0)
#define G_R_CG_SD 1.81
#define G_R_SD_CE 1.79
#define G_CB_CG_SD (-(PI - PI * 112.69 / 180.0))
#define G_CG_SD_CE (-(PI - PI * 100.61 / 180.0))
#define G_R_CG_CD2 1.35
#define G_R_CG_ND1 1.38
#define G_R_CG_NE2 2.1912
#define G_R_CG_CE1 2.1915
#define G_CB_CG_CD2 (-(PI - 2.27957453603))
#define G_CB_CG_ND1 (PI - 2.14413698608)
#define G_CB_CG_NE2 (-(PI - 2.90352974362))
#define G_CB_CG_CE1 (PI - 2.75209584734)

#define MAX_GROUP_ATOMS 10
#define MAX_SC_JOINTS 5

typedef struct {
    int chi;          /* 0..4 -> angle row 3+chi; -1 -> alpha fixed at 0 (Ala CB) */
    double beta, d;
    int natoms;
    const char *names[MAX_GROUP_ATOMS];
    double local[MAX_GROUP_ATOMS][3];
} ScJoint;

typedef struct {
    char letter;
    const char *name3;
    int natoms;                 /* heavy atoms, nUtil.cpp:192-517 (no OXT) */
    int njoints;                /* side-chain joints after the dummy transform */
    ScJoint j[MAX_SC_JOINTS];
    int pro;                    /* 1: CA group carries CB, CG, CD (cRigidGroup.cpp:165-172) */
} ResTemplate;

static ResTemplate T[20];
static int T_ready = 0;

static void set_atom(ScJoint *jt, int k, const char *name, double x, double y, double z) {
    jt->names[k] = name;
    jt->local[k][0] = x; jt->local[k][1] = y; jt->local[k][2] = z;
    if (k + 1 > jt->natoms) jt->natoms = k + 1;
}
static ScJoint joint(int chi, double beta, double d) {
    ScJoint j;
    memset(&j, 0, sizeof(j));
    j.chi = chi; j.beta = beta; j.d = d;
    return j;
}

/* Residue templates: cConformationAA.cpp:65-546 (joint order and parameters) and
 * cRigidGroup.cpp:30-210 (local atom positions). */
static void build_templates(void) {
    if (T_ready) return;
    memset(T, 0, sizeof(T));
    const double h = PI / 2.0;
    int n = 0;
    ResTemplate *r;
    ScJoint *j;
    double cv = cos(G_CA_CB_CG1 - h);

#define NEW(L3, l1, na) r = &T[n++]; r->letter = l1; r->name3 = L3; r->natoms = na; r->njoints = 0;
#define JOINT(chi, beta, d) j = &r->j[r->njoints++]; *j = joint(chi, beta, d);
    NEW("GLY", 'G', 4)
    NEW("ALA", 'A', 5)
    JOINT(-1, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    NEW("SER", 'S', 6)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    set_atom(j, 1, "OG", G_R_CB_OG * cos(-(PI - G_CA_CB_OG)), 0, G_R_CB_OG * sin(-(PI - G_CA_CB_OG)));
    NEW("CYS", 'C', 6)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    set_atom(j, 1, "SG", G_R_CB_SG * cos(-(PI - G_CA_CB_SG)), 0, G_R_CB_SG * sin(-(PI - G_CA_CB_SG)));
    NEW("VAL", 'V', 7)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    set_atom(j, 1, "CG1", G_R_CB_CG * sin(G_CA_CB_CG1 - h), G_R_CB_CG * cv * sin(G_CG1_CB_CG2 / 2.0), G_R_CB_CG * cv * cos(G_CG1_CB_CG2 / 2.0));
    set_atom(j, 2, "CG2", G_R_CB_CG * sin(G_CA_CB_CG1 - h), -G_R_CB_CG * cv * sin(G_CG1_CB_CG2 / 2.0), G_R_CB_CG * cv * cos(G_CG1_CB_CG2 / 2.0));
    NEW("ILE", 'I', 8)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    set_atom(j, 1, "CG2", G_R_CB_CG * sin(G_CA_CB_CG1 - h), G_R_CB_CG * cv * sin(G_CG1_CB_CG2), G_R_CB_CG * cv * cos(G_CG1_CB_CG2));
    JOINT(1, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CG1", 0, 0, 0);
    set_atom(j, 1, "CD1", G_R_CG1_CD1 * cos(PI - G_CB_CG1_CD1), 0, -G_R_CG1_CD1 * sin(PI - G_CB_CG1_CD1));
    NEW("LEU", 'L', 8)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "CD1", G_R_CB_CG * sin(G_CA_CB_CG1 - h), G_R_CB_CG * cv * sin(G_CG1_CB_CG2 / 2.0), G_R_CB_CG * cv * cos(G_CG1_CB_CG2 / 2.0));
    set_atom(j, 2, "CD2", G_R_CB_CG * sin(G_CA_CB_CG1 - h), -G_R_CB_CG * cv * sin(G_CG1_CB_CG2 / 2.0), G_R_CB_CG * cv * cos(G_CG1_CB_CG2 / 2.0));
    NEW("THR", 'T', 7)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    {
        double co = cos(G_CA_CB_OG1 - h);
        set_atom(j, 1, "OG1", G_R_CB_OG * sin(G_CA_CB_OG1 - h), G_R_CB_OG * co * sin(G_OG1_CB_CG2 / 2.0), G_R_CB_OG * co * cos(G_OG1_CB_CG2 / 2.0));
        set_atom(j, 2, "CG2", G_R_CB_CG * sin(G_CA_CB_CG1 - h), -G_R_CB_CG * cv * sin(G_OG1_CB_CG2 / 2.0), G_R_CB_CG * cv * cos(G_OG1_CB_CG2 / 2.0));
    }
    NEW("ARG", 'R', 11)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    JOINT(2, G_C_C_C, G_R_C_C) set_atom(j, 0, "CD", 0, 0, 0);
    JOINT(3, G_CG_CD_NE, G_R_CD_NE) set_atom(j, 0, "NE", 0, 0, 0);
    JOINT(4, G_CD_NE_CZ, G_R_NE_CZ) set_atom(j, 0, "CZ", 0, 0, 0);
    set_atom(j, 1, "NH1", G_R_CZ_NH * sin(G_NE_CZ_NH - h), 0, G_R_CZ_NH * cos(G_NE_CZ_NH - h));
    set_atom(j, 2, "NH2", G_R_CZ_NH * sin(G_NE_CZ_NH - h), 0, -G_R_CZ_NH * cos(G_NE_CZ_NH - h));
    NEW("LYS", 'K', 9)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    JOINT(2, G_C_C_C, G_R_C_C) set_atom(j, 0, "CD", 0, 0, 0);
    JOINT(3, G_C_C_C, G_R_CD_CE) set_atom(j, 0, "CE", 0, 0, 0);
    JOINT(4, G_CD_CE_NZ, G_R_CE_NZ) set_atom(j, 0, "NZ", 0, 0, 0);
    NEW("ASP", 'D', 8)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "OD1", G_R_CG_OD * sin(G_CB_CG_OD - h), 0, G_R_CG_OD * cos(G_CB_CG_OD - h));
    set_atom(j, 2, "OD2", G_R_CG_OD * sin(G_CB_CG_OD - h), 0, -G_R_CG_OD * cos(G_CB_CG_OD - h));
    NEW("ASN", 'N', 8)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "OD1", G_R_CG_OD1 * sin(G_CB_CG_OD1 - h), 0, G_R_CG_OD1 * cos(G_CB_CG_OD1 - h));
    set_atom(j, 2, "ND2", G_R_CG_ND2 * sin(G_CB_CG_ND2 - h), 0, -G_R_CG_ND2 * cos(G_CB_CG_ND2 - h));
    NEW("GLU", 'E', 9)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    JOINT(2, G_C_C_C, G_R_C_C) set_atom(j, 0, "CD", 0, 0, 0);
    set_atom(j, 1, "OE1", G_R_CG_OD * sin(G_CB_CG_OD - h), 0, G_R_CG_OD * cos(G_CB_CG_OD - h));
    set_atom(j, 2, "OE2", G_R_CG_OD * sin(G_CB_CG_OD - h), 0, -G_R_CG_OD * cos(G_CB_CG_OD - h));
    NEW("GLN", 'Q', 9)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    JOINT(2, G_C_C_C, G_R_C_C) set_atom(j, 0, "CD", 0, 0, 0);
    set_atom(j, 1, "OE1", G_R_CG_OD1 * sin(G_CB_CG_OD1 - h), 0, G_R_CG_OD1 * cos(G_CB_CG_OD1 - h));
    set_atom(j, 2, "NE2", G_R_CG_ND2 * sin(G_CB_CG_ND2 - h), 0, -G_R_CG_ND2 * cos(G_CB_CG_ND2 - h));
    NEW("MET", 'M', 8)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    JOINT(2, G_CB_CG_SD, G_R_CG_SD) set_atom(j, 0, "SD", 0, 0, 0);
    JOINT(3, G_CG_SD_CE, G_R_SD_CE) set_atom(j, 0, "CE", 0, 0, 0);
    NEW("HIS", 'H', 10)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "CD2", G_R_CG_CD2 * cos(G_CB_CG_CD2), G_R_CG_CD2 * sin(G_CB_CG_CD2), 0);
    set_atom(j, 2, "NE2", G_R_CG_NE2 * cos(G_CB_CG_NE2), G_R_CG_NE2 * sin(G_CB_CG_NE2), 0);
    set_atom(j, 3, "CE1", G_R_CG_CE1 * cos(G_CB_CG_CE1), G_R_CG_CE1 * sin(G_CB_CG_CE1), 0);
    set_atom(j, 4, "ND1", G_R_CG_ND1 * cos(G_CB_CG_ND1), G_R_CG_ND1 * sin(G_CB_CG_ND1), 0);
    NEW("PRO", 'P', 7)
    r->pro = 1;
    NEW("PHE", 'F', 11)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "CD1", 0.69229424, -1.20533343, 0);
    set_atom(j, 2, "CE1", 2.08228309, -1.20846014, 0);
    set_atom(j, 3, "CZ", 2.77997771, -0.00625341, 0);
    set_atom(j, 4, "CE2", 2.08768347, 1.19908002, 0);
    set_atom(j, 5, "CD2", 0.69769462, 1.20220673, 0);
    NEW("TYR", 'Y', 12)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "CD1", 0.69229424, -1.20533343, 0);
    set_atom(j, 2, "CE1", 2.08228309, -1.20846014, 0);
    set_atom(j, 3, "CZ", 2.77997771, -0.00625341, 0);
    set_atom(j, 4, "CE2", 2.08768347, 1.19908002, 0);
    set_atom(j, 5, "CD2", 0.69769462, 1.20220673, 0);
    set_atom(j, 6, "OH", 4.16960749, 0.05377697, 0);
    NEW("TRP", 'W', 14)
    JOINT(0, G_C_CA_CB, G_R_CA_CB) set_atom(j, 0, "CB", 0, 0, 0);
    JOINT(1, G_C_C_C, G_R_C_C) set_atom(j, 0, "CG", 0, 0, 0);
    set_atom(j, 1, "CD1", 0.829890578, -1.09003744, 0);
    set_atom(j, 2, "CD2", 0.84949676, 1.15028973, 0);
    set_atom(j, 3, "NE1", 2.1363699, -0.64570528, 0);
    set_atom(j, 4, "CE2", 2.18136443, 0.71889842, 0);
    set_atom(j, 5, "CE3", 0.61303306, 2.5301684, 0);
    set_atom(j, 6, "CZ2", 3.22086556, 1.65663275, 0);
    set_atom(j, 7, "CZ3", 1.68979906, 3.42486545, 0);
    set_atom(j, 8, "CH2", 2.92849902, 3.0257584, 0);
#undef NEW
#undef JOINT
    T_ready = 1;
}

static const ResTemplate *find_template(char c) {
    build_templates();
    for (int i = 0; i < 20; i++)
        if (T[i].letter == c) return &T[i];
    return NULL;
}

/* getSeqNumAtoms: nUtil.cpp:174-190 (add_terminal is always false). -1 on an unknown letter. */
int oracle_num_atoms(const char *seq) {
    int n = 0;
    for (const char *p = seq; *p; p++) {
        const ResTemplate *t = find_template(*p);
        if (!t) return -1;
        n += t->natoms;
    }
    return n;
}

/* ------------------------------------------------------ Angles2Coords tree */
typedef struct {
    int parent;
    int arow, acol;        /* alpha = angles[arow][acol]; arow < 0 -> alpha = aconst */
    double aconst, beta, d;
    int grow, gcol;        /* gradient slot; grow < 0 -> none */
    int natoms;
    int slot[MAX_GROUP_ATOMS];
    double local[MAX_GROUP_ATOMS][3];
    M44 M, F;
    int tin, tout;
} Node;

typedef struct {
    Node *nodes;
    int n, cap;
} Tree;

static int tree_add(Tree *t, int parent, int arow, int acol, double aconst, double beta, double d,
                    int grow, int gcol) {
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 256;
        t->nodes = (Node *)realloc(t->nodes, sizeof(Node) * t->cap);
    }
    Node *nd = &t->nodes[t->n];
    memset(nd, 0, sizeof(Node));
    nd->parent = parent; nd->arow = arow; nd->acol = acol; nd->aconst = aconst;
    nd->beta = beta; nd->d = d; nd->grow = grow; nd->gcol = gcol;
    return t->n++;
}
static void node_atom(Node *nd, int slot, const double *p) {
    nd->slot[nd->natoms] = slot;
    nd->local[nd->natoms][0] = p[0]; nd->local[nd->natoms][1] = p[1]; nd->local[nd->natoms][2] = p[2];
    nd->natoms++;
}

/* Graph of one chain, cConformation.cpp:30-131 with the templates of cConformationAA.cpp. */
static int build_tree(Tree *t, const char *seq, int len) {
    static const double zero[3] = {0, 0, 0};
    int lastC = -1, first = 0;
    for (int i = 0; i < len; i++) {
        const ResTemplate *r = find_template(seq[i]);
        if (!r) return -1;
        int nN;
        if (lastC < 0) nN = tree_add(t, -1, -1, 0, 0.0, 0.0, 0.0, -1, 0);
        else nN = tree_add(t, lastC, 2, i - 1, 0.0, G_CA_C_N, R_C_N, 2, i - 1);
        node_atom(&t->nodes[nN], first + 0, zero);
        int nCA = tree_add(t, nN, 0, i, 0.0, G_C_N_CA, R_N_CA, 0, i);
        node_atom(&t->nodes[nCA], first + 1, zero);
        if (r->pro) {
            const double cb[3] = {0.36842372, -1.29540981, 0.70468246};
            const double cg[3] = {-0.76137817, -2.21546205, 0.39299099};
            const double cd[3] = {-1.97838492, -1.33927458, 0.35849352};
            node_atom(&t->nodes[nCA], first + 2, cb);
            node_atom(&t->nodes[nCA], first + 3, cg);
            node_atom(&t->nodes[nCA], first + 4, cd);
        }
        if (r->njoints > 0) {
            int parent = tree_add(t, nCA, -1, 0, G_N_C_CA_CB, 0.0, 0.0, -1, 0); /* dummy */
            int slot = first + 2;
            for (int k = 0; k < r->njoints; k++) {
                const ScJoint *jt = &r->j[k];
                int nd;
                if (jt->chi < 0) nd = tree_add(t, parent, -1, 0, 0.0, jt->beta, jt->d, -1, 0);
                else nd = tree_add(t, parent, 3 + jt->chi, i, 0.0, jt->beta, jt->d, 3 + jt->chi, i);
                for (int a = 0; a < jt->natoms; a++) node_atom(&t->nodes[nd], slot++, jt->local[a]);
                parent = nd;
            }
        }
        int nC = tree_add(t, nCA, 1, i, 0.0, G_N_CA_C, R_CA_C, 1, i);
        const double o[3] = {G_R_CB_OG * cos(G_CA_C_O), 0.0, G_R_CB_OG * sin(G_CA_C_O)};
        node_atom(&t->nodes[nC], first + r->natoms - 2, zero);
        node_atom(&t->nodes[nC], first + r->natoms - 1, o);
        lastC = nC;
        first += r->natoms;
    }
    return first;
}

static int seq_length(const unsigned char *s, int stride) {
    int n = 0;
    while (n < stride && s[n]) n++;
    return n;
}

/* cConformation::update (cConformation.cpp:160-178); nodes are stored parent-first. */
static void tree_forward(Tree *t, const double *ang, int L) {
    for (int k = 0; k < t->n; k++) {
        Node *nd = &t->nodes[k];
        double alpha = nd->arow < 0 ? nd->aconst : ang[(size_t)nd->arow * L + nd->acol];
        M44 mat, dmat, inv;
        joint_matrices(alpha, nd->beta, nd->d, &mat, &dmat);
        if (nd->parent < 0) {
            m44_identity(&nd->M);
            inv = m44_rigid_inverse(&nd->M);
            nd->F = m44_mul(&dmat, &inv);
        } else {
            const M44 *P = &t->nodes[nd->parent].M;
            nd->M = m44_mul(P, &mat);
            M44 left = m44_mul(P, &dmat);
            inv = m44_rigid_inverse(&nd->M);
            nd->F = m44_mul(&left, &inv);
        }
    }
}

static const char *atom_name_of(const ResTemplate *r, int k) {
    /* k = offset inside the residue */
    static const char *pro[] = {"N", "CA", "CB", "CG", "CD", "C", "O"};
    if (r->pro) return pro[k];
    if (k == 0) return "N";
    if (k == 1) return "CA";
    if (k == r->natoms - 2) return "C";
    if (k == r->natoms - 1) return "O";
    int s = 2;
    for (int jn = 0; jn < r->njoints; jn++)
        for (int a = 0; a < r->j[jn].natoms; a++, s++)
            if (s == k) return r->j[jn].names[a];
    return "?";
}

int oracle_a2c_forward(const unsigned char *seqs, int seq_stride, const double *angles,
                       double *coords, unsigned char *res_names, unsigned char *atom_names,
                       int B, int L, int maxA) {
    build_templates();
    for (int b = 0; b < B; b++) {
        const unsigned char *s = seqs + (size_t)b * seq_stride;
        int len = seq_length(s, seq_stride);
        if (len > L) return -2;
        Tree t = {0};
        int na = build_tree(&t, (const char *)s, len);
        if (na < 0) { free(t.nodes); return -3; }
        if (na > maxA) { free(t.nodes); return -4; }
        const double *ang = angles + (size_t)b * 8 * L;
        double *x = coords + (size_t)b * 3 * maxA;
        memset(x, 0, sizeof(double) * 3 * maxA);
        tree_forward(&t, ang, L);
        for (int k = 0; k < t.n; k++) {
            Node *nd = &t.nodes[k];
            for (int a = 0; a < nd->natoms; a++) m44_apply(&nd->M, nd->local[a], x + 3 * nd->slot[a]);
        }
        if (res_names && atom_names) {
            unsigned char *rn = res_names + (size_t)b * maxA * 4;
            unsigned char *an = atom_names + (size_t)b * maxA * 4;
            memset(rn, 0, (size_t)maxA * 4);
            memset(an, 0, (size_t)maxA * 4);
            int slot = 0;
            for (int i = 0; i < len; i++) {
                const ResTemplate *r = find_template((char)s[i]);
                for (int k = 0; k < r->natoms; k++, slot++) {
                    memcpy(rn + 4 * slot, r->name3, 3);
                    const char *nm = atom_name_of(r, k);
                    memcpy(an + 4 * slot, nm, strlen(nm));
                }
            }
        }
        free(t.nodes);
    }
    return 0;
}

/* cConformation::backward (cConformation.cpp:180-211): O(nodes x subtree). */
int oracle_a2c_backward(const double *grad_coords, double *grad_angles, const unsigned char *seqs,
                        int seq_stride, const double *angles, int B, int L, int maxA) {
    build_templates();
    for (int b = 0; b < B; b++) {
        const unsigned char *s = seqs + (size_t)b * seq_stride;
        int len = seq_length(s, seq_stride);
        double *ga = grad_angles + (size_t)b * 8 * L;
        for (int k = 0; k < 8 * L; k++) ga[k] = 0.0;
        if (len > L) return -2;
        Tree t = {0};
        int na = build_tree(&t, (const char *)s, len);
        if (na < 0) { free(t.nodes); return -3; }
        if (na > maxA) { free(t.nodes); return -4; }
        const double *ang = angles + (size_t)b * 8 * L;
        const double *g = grad_coords + (size_t)b * 3 * maxA;
        tree_forward(&t, ang, L);
        /* global atom positions */
        double *x = (double *)malloc(sizeof(double) * 3 * (na > 0 ? na : 1));
        for (int k = 0; k < t.n; k++) {
            Node *nd = &t.nodes[k];
            for (int a = 0; a < nd->natoms; a++) m44_apply(&nd->M, nd->local[a], x + 3 * nd->slot[a]);
        }
        /* subtree intervals by DFS over children (children in creation order) */
        int *first_child = (int *)malloc(sizeof(int) * t.n), *next_sib = (int *)malloc(sizeof(int) * t.n);
        int *stack = (int *)malloc(sizeof(int) * (t.n + 1)), *order = (int *)malloc(sizeof(int) * t.n);
        int *last_child = (int *)malloc(sizeof(int) * t.n);
        for (int k = 0; k < t.n; k++) first_child[k] = next_sib[k] = last_child[k] = -1;
        for (int k = 1; k < t.n; k++) {
            int p = t.nodes[k].parent;
            if (first_child[p] < 0) first_child[p] = k; else next_sib[last_child[p]] = k;
            last_child[p] = k;
        }
        int sp = 0, cnt = 0;
        if (t.n > 0) stack[sp++] = 0;
        /* iterative pre-order; tout = tin + subtree size */
        while (sp) {
            int k = stack[--sp];
            t.nodes[k].tin = cnt;
            order[cnt++] = k;
            /* push children in reverse so the first child is visited first */
            int tmp[8], nc = 0;
            for (int c = first_child[k]; c >= 0; c = next_sib[c]) tmp[nc++] = c;
            while (nc) stack[sp++] = tmp[--nc];
        }
        for (int q = t.n - 1; q >= 0; q--) {
            int k = order[q];
            int end = t.nodes[k].tin + 1;
            for (int c = first_child[k]; c >= 0; c = next_sib[c])
                if (t.nodes[c].tout > end) end = t.nodes[c].tout;
            t.nodes[k].tout = end;
        }
        for (int k = 0; k < t.n; k++) {
            Node *nd = &t.nodes[k];
            if (nd->grow < 0) continue;
            double sum = 0.0;
            for (int q = nd->tin; q < nd->tout; q++) {
                Node *sub = &t.nodes[order[q]];
                for (int a = 0; a < sub->natoms; a++) {
                    double f[3];
                    int sl = sub->slot[a];
                    m44_apply(&nd->F, x + 3 * sl, f);
                    sum += g[3 * sl] * f[0] + g[3 * sl + 1] * f[1] + g[3 * sl + 2] * f[2];
                }
            }
            ga[(size_t)nd->grow * L + nd->gcol] = sum;
        }
        free(x); free(first_child); free(next_sib); free(stack); free(order); free(last_child);
        free(t.nodes);
    }
    return 0;
}
