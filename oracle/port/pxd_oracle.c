/*
 * pxd_oracle.c -- TEST INFRASTRUCTURE: FP64 C restatement of the reference hot path.
 * See pxd_oracle.h. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg use this file; it is the checker, never the product.
 */
#define _GNU_SOURCE
#include "pxd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/pxdock_gb300_vdw.h"

#define EPS 1e-20 /* kParamEpsilon, math.h:128 */
static const double kCoulomb = 332.0637141491396; /* kCoulombFactor, system.h:83 */
static const double kPi = 3.141592653589793;      /* kMathPi, math.h:224 */

/* ------------------------------------------------------------ small vectors */
static inline void v_sub(const double* a, const double* b, double* c) {
    c[0] = a[0] - b[0];
    c[1] = a[1] - b[1];
    c[2] = a[2] - b[2];
}
static inline void v_add(const double* a, const double* b, double* c) {
    c[0] = a[0] + b[0];
    c[1] = a[1] + b[1];
    c[2] = a[2] + b[2];
}
static inline void v_addi(double* a, const double* b) {
    a[0] += b[0];
    a[1] += b[1];
    a[2] += b[2];
}
static inline void v_subi(double* a, const double* b) {
    a[0] -= b[0];
    a[1] -= b[1];
    a[2] -= b[2];
}
static inline void v_scale(const double* a, double f, double* c) {
    c[0] = a[0] * f;
    c[1] = a[1] * f;
    c[2] = a[2] * f;
}
static inline void v_scalei(double* a, double f) {
    a[0] *= f;
    a[1] *= f;
    a[2] *= f;
}
static inline double v_dot(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline double v_sqsum(const double* a) {
    double s = a[0] * a[0];
    s += a[1] * a[1];
    s += a[2] * a[2];
    return s;
}
static inline double v_norm(const double* a) { return sqrt(v_sqsum(a)); }
static inline void v_cross(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static inline void v_normalize(double* a) {
    double n = v_norm(a);
    a[0] /= n;
    a[1] /= n;
    a[2] /= n;
}
static inline void m_apply(const double* m, const double* v, double* out) {
    out[0] = v_dot(m, v);
    out[1] = v_dot(m + 3, v);
    out[2] = v_dot(m + 6, v);
}
static inline void m_mul(const double* r, const double* s, double* o) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            o[3 * i + j] = r[3 * i] * s[j] + r[3 * i + 1] * s[3 + j] + r[3 * i + 2] * s[6 + j];
}
static inline double safe_div(double a, double b) { return a / (b + EPS); }

/* ------------------------------------------------------------- math.cpp:22-167 */
void po_rotation_quaternion(const double* q, double* m) {
    const double aa = q[0] * q[0], ab = q[0] * q[1], ac = q[0] * q[2], ad = q[0] * q[3];
    const double bb = q[1] * q[1], bc = q[1] * q[2], bd = q[1] * q[3];
    const double cc = q[2] * q[2], cd = q[2] * q[3], dd = q[3] * q[3];
    m[0] = aa + bb - cc - dd;
    m[1] = 2 * (bc - ad);
    m[2] = 2 * (ac + bd);
    m[3] = 2 * (ad + bc);
    m[4] = aa - bb + cc - dd;
    m[5] = 2 * (cd - ab);
    m[6] = 2 * (bd - ac);
    m[7] = 2 * (ab + cd);
    m[8] = aa - bb - cc + dd;
}

/* Rodrigues matrix about a unit axis (math.cpp:44-60). */
static void rotation_axis_angle(const double* k, double theta, double* m) {
    const double st = sin(theta), ct = cos(theta), omc = 1 - ct;
    m[0] = ct + k[0] * k[0] * omc;
    m[1] = k[0] * k[1] * omc - k[2] * st;
    m[2] = k[1] * st + k[0] * k[2] * omc;
    m[3] = k[2] * st + k[0] * k[1] * omc;
    m[4] = ct + k[1] * k[1] * omc;
    m[5] = k[1] * k[2] * omc - k[0] * st;
    m[6] = k[0] * k[2] * omc - k[1] * st;
    m[7] = k[0] * st + k[1] * k[2] * omc;
    m[8] = ct + k[2] * k[2] * omc;
}

/* Rodrigues matrix and its theta-derivative (math.cpp:62-94). */
void po_rotation_axis_angle(const double* k, double theta, double* m, double* j) {
    const double st = sin(theta), ct = cos(theta), omc = 1 - ct;
    const double kxo = k[0] * omc, kyo = k[1] * omc, kzo = k[2] * omc;
    const double kxs = k[0] * st, kys = k[1] * st, kzs = k[2] * st;
    m[0] = ct + k[0] * kxo;
    m[1] = k[1] * kxo - kzs;
    m[2] = kys + k[2] * kxo;
    m[3] = kzs + k[0] * kyo;
    m[4] = ct + k[1] * kyo;
    m[5] = k[2] * kyo - kxs;
    m[6] = k[0] * kzo - kys;
    m[7] = kxs + k[1] * kzo;
    m[8] = ct + k[2] * kzo;
    j[0] = -st + k[0] * kxs;
    j[1] = -k[2] * ct + k[0] * kys;
    j[2] = k[1] * ct + k[0] * kzs;
    j[3] = k[2] * ct + k[1] * kxs;
    j[4] = -st + k[1] * kys;
    j[5] = -k[0] * ct + k[1] * kzs;
    j[6] = -k[1] * ct + k[2] * kxs;
    j[7] = k[0] * ct + k[2] * kys;
    j[8] = -st + k[2] * kzs;
}

/* Bond angle at j and its gradient on i and k (math.cpp:96-110). */
double po_angle_and_gradient(const double* pi, const double* pj, const double* pk, double* gi,
                             double* gk) {
    double v0[3], v1[3], c[3];
    v_sub(pj, pi, v0);
    v_sub(pj, pk, v1);
    v_cross(v0, v1, c);
    const double rp = v_norm(c);
    v_cross(v0, c, gi);
    v_cross(c, v1, gk);
    v_scalei(gi, -safe_div(1.0, v_sqsum(v0) * rp));
    v_scalei(gk, -safe_div(1.0, v_sqsum(v1) * rp));
    return atan2(rp, v_dot(v0, v1) + EPS);
}

/* Signed dihedral angle (math.cpp:112-128). */
double po_dihedral(const double* pi, const double* pj, const double* pk, const double* pl) {
    double rij[3], rkj[3], w[3], m[3], n[3];
    v_sub(pj, pi, rij);
    v_sub(pj, pk, rkj);
    v_sub(pl, pk, w);
    v_cross(rij, rkj, m);
    v_cross(rkj, w, n);
    v_cross(m, n, w);
    const double wlen = v_norm(w);
    const double s = v_dot(m, n);
    const double phi = atan2(wlen, s + EPS);
    const double ipr = v_dot(rij, n);
    return ipr < 0.0 ? phi : -phi;
}

/* Dihedral angle and its gradient on the four atoms (math.cpp:130-167). */
double po_dihedral_and_gradient(const double* pi, const double* pj, const double* pk,
                                const double* pl, double* gi, double* gj, double* gk,
                                double* gl) {
    double rij[3], rkj[3], rkl[3], m[3], n[3], w[3];
    v_sub(pj, pi, rij);
    v_sub(pj, pk, rkj);
    v_sub(pl, pk, rkl);
    v_cross(rij, rkj, m);
    v_cross(rkj, rkl, n);
    v_cross(m, n, w);
    const double wlen = v_norm(w);
    const double s = v_dot(m, n);
    const double phi = atan2(wlen, s + EPS);
    const double ipr = v_dot(rij, n);
    const double theta = ipr < 0.0 ? phi : -phi;
    const double nrkj2 = v_sqsum(rkj);
    const double nrkj_1 = safe_div(1.0, sqrt(nrkj2));
    const double nrkj_2 = nrkj_1 * nrkj_1;
    const double nrkj = nrkj2 * nrkj_1;
    const double a = -nrkj / v_sqsum(m);
    const double b = nrkj / v_sqsum(n);
    v_scale(m, -a, gi);
    v_scale(n, -b, gl);
    const double p = v_dot(rij, rkj) * nrkj_2;
    const double q = v_dot(rkj, rkl) * nrkj_2;
    double uvec[3], vvec[3], svec[3];
    v_scale(gi, p, uvec);
    v_scale(gl, q, vvec);
    v_sub(uvec, vvec, svec);
    v_sub(gi, svec, gj);
    v_add(gl, svec, gk);
    v_scalei(gj, -1.0);
    v_scalei(gk, -1.0);
    return theta;
}

void po_vdw_type_table(double* sigma, double* epsilon) {
    for (int i = 0; i < PXD_NUM_VDW_TYPES; ++i) {
        sigma[i] = PXD_VDW_SIGMA[i];
        epsilon[i] = PXD_VDW_EPSILON[i];
    }
}

/* ------------------------------------------------------------- pair.h:25-60 */
static inline double coul_pair(double qi, double qj, const double* rij, double d, double scale,
                               double* gi, double* gj) {
    const double qq = qi * qj * scale;
    const double de_dr_r = -safe_div(qq, d * d * d) * kCoulomb;
    double g[3];
    v_scale(rij, de_dr_r, g);
    v_subi(gi, g);
    v_addi(gj, g);
    return safe_div(qq, d) * kCoulomb;
}

static inline double vdw_pair(double si, double ei, double sj, double ej, const double* rij,
                              double d, double scale, double* gi, double* gj) {
    double fused = (si + sj) * 0.5;
    const double u6 = pow(safe_div(fused, d), 6.0);
    const double u12 = u6 * u6;
    fused = sqrt(ei * ej) * scale * 4.0;
    const double irsqr = safe_div(1.0, d * d);
    const double de_dr_r = (-12.0 * u12 + 6.0 * u6) * irsqr * fused;
    double g[3];
    v_scale(rij, de_dr_r, g);
    v_subi(gi, g);
    v_addi(gj, g);
    return (u12 - u6) * fused;
}

/* ------------------------------------------------- interaction.cpp:27-196 */
static double bonds_energy(const pxd_topology* ff, const double* x, double* g) {
    double e = 0.0;
    for (int b = 0; b < ff->n_bonds; ++b) {
        const int i = ff->bond_atoms[2 * b], j = ff->bond_atoms[2 * b + 1];
        double d[3];
        v_sub(x + 3 * j, x + 3 * i, d);
        const double r = v_norm(d);
        const double dr = r - ff->bond_length[b];
        e += 0.5 * ff->bond_k[b] * (dr * dr);
        const double de_dr = ff->bond_k[b] * (1 - safe_div(ff->bond_length[b], r));
        v_scalei(d, de_dr);
        v_subi(g + 3 * i, d);
        v_addi(g + 3 * j, d);
    }
    return e;
}

static double angles_energy(const pxd_topology* ff, const double* x, double* g) {
    double e = 0.0;
    for (int a = 0; a < ff->n_angles; ++a) {
        const int i = ff->angle_atoms[3 * a], j = ff->angle_atoms[3 * a + 1],
                  k = ff->angle_atoms[3 * a + 2];
        double fi[3], fk[3], fj[3];
        const double theta = po_angle_and_gradient(x + 3 * i, x + 3 * j, x + 3 * k, fi, fk);
        const double delta = theta - ff->angle_radian[a];
        e += 0.5 * ff->angle_k[a] * (delta * delta);
        const double de_dt = ff->angle_k[a] * delta;
        v_scalei(fi, de_dt);
        v_scalei(fk, de_dt);
        v_addi(g + 3 * i, fi);
        v_addi(g + 3 * k, fk);
        v_add(fi, fk, fj);
        v_subi(g + 3 * j, fj);
    }
    return e;
}

static double one_dihedral(const int32_t* ids, const int32_t* per, const double* phase,
                           const double* kk, const double* x, double* g) {
    const int i = ids[0], j = ids[1], k = ids[2], l = ids[3];
    double gi[3], gj[3], gk[3], gl[3], gg[3];
    const double theta =
        po_dihedral_and_gradient(x + 3 * i, x + 3 * j, x + 3 * k, x + 3 * l, gi, gj, gk, gl);
    double e = 0.0;
    for (int t = 0; t < 6; ++t) {
        if (per[t] == 0) break;
        const double delta = theta * per[t] - phase[t];
        e += kk[t] * (1 + cos(delta));
        const double de_dt = kk[t] * per[t] * sin(delta);
        v_scale(gi, -de_dt, gg);
        v_addi(g + 3 * i, gg);
        v_scale(gj, -de_dt, gg);
        v_addi(g + 3 * j, gg);
        v_scale(gk, -de_dt, gg);
        v_addi(g + 3 * k, gg);
        v_scale(gl, -de_dt, gg);
        v_addi(g + 3 * l, gg);
    }
    return e;
}

static double dihedrals_energy(const pxd_topology* ff, const double* x, double* g) {
    double e = 0.0;
    for (int d = 0; d < ff->n_impropers; ++d)
        e += one_dihedral(ff->improper_atoms + 4 * d, ff->improper_periodicity + 6 * d,
                          ff->improper_phase + 6 * d, ff->improper_k + 6 * d, x, g);
    for (int d = 0; d < ff->n_propers; ++d)
        e += one_dihedral(ff->proper_atoms + 4 * d, ff->proper_periodicity + 6 * d,
                          ff->proper_phase + 6 * d, ff->proper_k + 6 * d, x, g);
    return e;
}

static double nonbonded_energy(const pxd_topology* ff, const double* x, double* g) {
    const double coul14 = 0.833333333, vdw14 = 0.5; /* interaction.h:52-53 */
    double e1 = 0.0, e2 = 0.0;
    for (int p = 0; p < ff->n_pairs14; ++p) {
        const int i = ff->pairs14[2 * p], j = ff->pairs14[2 * p + 1];
        double rij[3];
        v_sub(x + 3 * j, x + 3 * i, rij);
        const double d = v_norm(rij);
        e1 += coul_pair(ff->charge[i], ff->charge[j], rij, d, coul14, g + 3 * i, g + 3 * j);
        e2 += vdw_pair(ff->sigma[i], ff->epsilon[i], ff->sigma[j], ff->epsilon[j], rij, d, vdw14,
                       g + 3 * i, g + 3 * j);
    }
    for (int p = 0; p < ff->n_pairs; ++p) {
        const int i = ff->pairs[2 * p], j = ff->pairs[2 * p + 1];
        double rij[3];
        v_sub(x + 3 * j, x + 3 * i, rij);
        const double d = v_norm(rij);
        e1 += coul_pair(ff->charge[i], ff->charge[j], rij, d, 1.0, g + 3 * i, g + 3 * j);
        e2 += vdw_pair(ff->sigma[i], ff->epsilon[i], ff->sigma[j], ff->epsilon[j], rij, d, 1.0,
                       g + 3 * i, g + 3 * j);
    }
    return e1 + e2;
}

double po_intra_energy(int which, const pxd_topology* ff, const double* x, double* g) {
    switch (which) {
        case 0: return bonds_energy(ff, x, g);
        case 1: return angles_energy(ff, x, g);
        case 2: return dihedrals_energy(ff, x, g);
        case 3: return nonbonded_energy(ff, x, g);
        default: {
            double e = 0.0;
            e += bonds_energy(ff, x, g);
            e += angles_energy(ff, x, g);
            e += dihedrals_energy(ff, x, g);
            e += nonbonded_energy(ff, x, g);
            return e;
        }
    }
}

/* ----------------------------------------------------------- owned copies */
typedef struct {
    pxd_topology t;
    void* blocks[32];
    int nblocks;
} owned_topology;

static void* dup_block(owned_topology* o, const void* src, size_t bytes) {
    if (!src || bytes == 0) return NULL;
    void* p = malloc(bytes);
    memcpy(p, src, bytes);
    o->blocks[o->nblocks++] = p;
    return p;
}

static void own_topology(owned_topology* o, const pxd_topology* t) {
    memset(o, 0, sizeof(*o));
    o->t = *t;
    const size_t n = (size_t)t->n_atoms;
    o->t.charge = dup_block(o, t->charge, n * sizeof(double));
    o->t.sigma = dup_block(o, t->sigma, n * sizeof(double));
    o->t.epsilon = dup_block(o, t->epsilon, n * sizeof(double));
    o->t.bond_atoms = dup_block(o, t->bond_atoms, (size_t)t->n_bonds * 2 * sizeof(int32_t));
    o->t.bond_k = dup_block(o, t->bond_k, (size_t)t->n_bonds * sizeof(double));
    o->t.bond_length = dup_block(o, t->bond_length, (size_t)t->n_bonds * sizeof(double));
    o->t.angle_atoms = dup_block(o, t->angle_atoms, (size_t)t->n_angles * 3 * sizeof(int32_t));
    o->t.angle_k = dup_block(o, t->angle_k, (size_t)t->n_angles * sizeof(double));
    o->t.angle_radian = dup_block(o, t->angle_radian, (size_t)t->n_angles * sizeof(double));
    o->t.improper_atoms =
        dup_block(o, t->improper_atoms, (size_t)t->n_impropers * 4 * sizeof(int32_t));
    o->t.improper_periodicity =
        dup_block(o, t->improper_periodicity, (size_t)t->n_impropers * 6 * sizeof(int32_t));
    o->t.improper_phase =
        dup_block(o, t->improper_phase, (size_t)t->n_impropers * 6 * sizeof(double));
    o->t.improper_k = dup_block(o, t->improper_k, (size_t)t->n_impropers * 6 * sizeof(double));
    o->t.proper_atoms = dup_block(o, t->proper_atoms, (size_t)t->n_propers * 4 * sizeof(int32_t));
    o->t.proper_periodicity =
        dup_block(o, t->proper_periodicity, (size_t)t->n_propers * 6 * sizeof(int32_t));
    o->t.proper_phase = dup_block(o, t->proper_phase, (size_t)t->n_propers * 6 * sizeof(double));
    o->t.proper_k = dup_block(o, t->proper_k, (size_t)t->n_propers * 6 * sizeof(double));
    o->t.pairs14 = dup_block(o, t->pairs14, (size_t)t->n_pairs14 * 2 * sizeof(int32_t));
    o->t.pairs = dup_block(o, t->pairs, (size_t)t->n_pairs * 2 * sizeof(int32_t));
}

static void free_topology(owned_topology* o) {
    for (int i = 0; i < o->nblocks; ++i) free(o->blocks[i]);
    o->nblocks = 0;
}

/* ---------------------------------------------------------------- system */
struct po_system {
    /* receptor */
    int n_rec;
    double* rec_xyz0;    /* [n_rec][3] input coordinates */
    owned_topology rec;
    int n_rotors;
    double* rotor_origin; /* [n_rotors][3] axis_origin */
    double* rotor_axis;   /* [n_rotors][3] unit axis_vector */
    int* mov_offsets;     /* [n_rotors+1] */
    int* mov_atoms;       /* movable atoms, axis atom removed (data.cpp:358-361) */
    int n_mov;
    unsigned char* excluded; /* [n_rec] 1 for movable atoms */
    int* excl_list;          /* sorted movable atoms (grid.cpp:118-123) */
    int n_excl;
    /* ligand */
    int n_lig;
    owned_topology lig;
    int* lig_type;
    /* torsion tree */
    int n_frags, n_roots, n_tors;
    int *frag_start, *frag_end, *perm, *rev, *roots;
    int *tors_frag, *tors_parent, *tors_parent_atom, *tors_mine_atom;
    int* frag_children_off; /* CSR of children per fragment, pre-order listing */
    int* frag_children;
    /* grid */
    int has_grid;
    pxd_box box;
    double spacing_inv;
    int npm1[3];
    double slope;
    double* maps[PXD_NUM_VDW_TYPES + 1]; /* [P][4] each; index 99 = Coulomb */
};

static int* dup_ints(const int32_t* src, size_t n) {
    int* p = (int*)malloc((n ? n : 1) * sizeof(int));
    for (size_t i = 0; i < n; ++i) p[i] = src[i];
    return p;
}

po_system* po_system_create(const pxd_receptor_desc* rec, const pxd_ligand_desc* lig) {
    po_system* s = (po_system*)calloc(1, sizeof(po_system));
    /* receptor: torsional_receptor::parse post-processing (data.cpp:349-363) */
    s->n_rec = rec->n_atoms;
    s->rec_xyz0 = (double*)malloc((size_t)(s->n_rec ? s->n_rec : 1) * 3 * sizeof(double));
    memcpy(s->rec_xyz0, rec->xyz, (size_t)s->n_rec * 3 * sizeof(double));
    own_topology(&s->rec, &rec->ff);
    s->n_rotors = rec->n_rotors;
    s->rotor_origin = (double*)malloc((size_t)(s->n_rotors + 1) * 3 * sizeof(double));
    s->rotor_axis = (double*)malloc((size_t)(s->n_rotors + 1) * 3 * sizeof(double));
    s->mov_offsets = (int*)malloc((size_t)(s->n_rotors + 1) * sizeof(int));
    const int total = s->n_rotors ? rec->rotor_offsets[s->n_rotors] : 0;
    s->mov_atoms = (int*)malloc((size_t)(total + 1) * sizeof(int));
    s->excluded = (unsigned char*)calloc((size_t)(s->n_rec + 1), 1);
    s->n_mov = 0;
    for (int r = 0; r < s->n_rotors; ++r) {
        const int a0 = rec->rotor_axis[2 * r], a1 = rec->rotor_axis[2 * r + 1];
        memcpy(s->rotor_origin + 3 * r, rec->xyz + 3 * a0, 3 * sizeof(double));
        v_sub(rec->xyz + 3 * a1, s->rotor_origin + 3 * r, s->rotor_axis + 3 * r);
        v_normalize(s->rotor_axis + 3 * r);
        s->mov_offsets[r] = s->n_mov;
        for (int k = rec->rotor_offsets[r]; k < rec->rotor_offsets[r + 1]; ++k) {
            const int j = rec->rotor_atoms[k];
            if (j != a1) {
                s->mov_atoms[s->n_mov++] = j;
                s->excluded[j] = 1;
            }
        }
    }
    s->mov_offsets[s->n_rotors] = s->n_mov;
    s->excl_list = (int*)malloc((size_t)(s->n_mov + 1) * sizeof(int));
    s->n_excl = 0;
    for (int j = 0; j < s->n_rec; ++j)
        if (s->excluded[j]) s->excl_list[s->n_excl++] = j;
    /* ligand */
    s->n_lig = lig->ff.n_atoms;
    own_topology(&s->lig, &lig->ff);
    s->lig_type = dup_ints(lig->vdw_type, (size_t)s->n_lig);
    /* torsion tree (data.cpp:410-482 in flat form) */
    const pxd_torsion_tree* t = &lig->tree;
    s->n_frags = t->n_frags;
    s->n_roots = t->n_roots;
    s->n_tors = t->n_torsions;
    if (t->n_frags > 0) {
        s->frag_start = dup_ints(t->frag_start, (size_t)t->n_frags);
        s->frag_end = dup_ints(t->frag_end, (size_t)t->n_frags);
        s->perm = dup_ints(t->perm, (size_t)s->n_lig);
        s->rev = (int*)malloc((size_t)(s->n_lig + 1) * sizeof(int));
        for (int p = 0; p < s->n_lig; ++p) s->rev[s->perm[p]] = p;
        s->roots = dup_ints(t->roots, (size_t)t->n_roots);
        s->tors_frag = dup_ints(t->tors_frag, (size_t)t->n_torsions);
        s->tors_parent = dup_ints(t->tors_parent, (size_t)t->n_torsions);
        s->tors_parent_atom = dup_ints(t->tors_parent_atom, (size_t)t->n_torsions);
        s->tors_mine_atom = dup_ints(t->tors_mine_atom, (size_t)t->n_torsions);
    }
    s->slope = 0.0;
    return s;
}

void po_system_destroy(po_system* s) {
    if (!s) return;
    po_drop_grid(s);
    free(s->rec_xyz0);
    free_topology(&s->rec);
    free(s->rotor_origin);
    free(s->rotor_axis);
    free(s->mov_offsets);
    free(s->mov_atoms);
    free(s->excluded);
    free(s->excl_list);
    free_topology(&s->lig);
    free(s->lig_type);
    free(s->frag_start);
    free(s->frag_end);
    free(s->perm);
    free(s->rev);
    free(s->roots);
    free(s->tors_frag);
    free(s->tors_parent);
    free(s->tors_parent_atom);
    free(s->tors_mine_atom);
    free(s);
}

/* ------------------------------------------------------------ grid (grid.cpp) */
typedef struct {
    po_system* s;
    const int* types;
    int n_types;
    int i0, i1;
} grid_job;

/* partial_worker::populate (grid.cpp:150-195) for the i-slab [i0, i1). */
static void* grid_worker(void* arg) {
    grid_job* job = (grid_job*)arg;
    po_system* s = job->s;
    const pxd_box* bc = &s->box;
    const int ny = bc->npoints[1], nz = bc->npoints[2];
    double point[3], vec[3], tmp[3];
    double* acc = (double*)malloc((size_t)(job->n_types + 1) * 4 * sizeof(double));
    for (int i = job->i0; i < job->i1; ++i) {
        point[0] = bc->init_xyz[0] + bc->spacing * i;
        for (int j = 0; j < ny; ++j) {
            point[1] = bc->init_xyz[1] + bc->spacing * j;
            for (int k = 0; k < nz; ++k) {
                point[2] = bc->init_xyz[2] + bc->spacing * k;
                memset(acc, 0, (size_t)(job->n_types + 1) * 4 * sizeof(double));
                for (int a = 0; a < s->n_rec; ++a) {
                    if (s->excluded[a]) continue;
                    v_sub(s->rec_xyz0 + 3 * a, point, vec);
                    const double d = v_norm(vec);
                    acc[0] += coul_pair(1.0, s->rec.t.charge[a], vec, d, 1.0, acc + 1, tmp);
                    for (int t = 0; t < job->n_types; ++t) {
                        const int ty = job->types[t];
                        double* at = acc + 4 * (t + 1);
                        at[0] += vdw_pair(PXD_VDW_SIGMA[ty], PXD_VDW_EPSILON[ty], s->rec.t.sigma[a],
                                          s->rec.t.epsilon[a], vec, d, 1.0, at + 1, tmp);
                    }
                }
                const size_t off = ((size_t)i * ny + j) * nz + k;
                memcpy(s->maps[PXD_NUM_VDW_TYPES] + 4 * off, acc, 4 * sizeof(double));
                for (int t = 0; t < job->n_types; ++t)
                    memcpy(s->maps[job->types[t]] + 4 * off, acc + 4 * (t + 1), 4 * sizeof(double));
            }
        }
    }
    free(acc);
    return NULL;
}

int po_build_grid(po_system* s, const pxd_box* box, const int32_t* types, int32_t n_types,
                  int nthreads) {
    po_drop_grid(s);
    s->box = *box;
    s->spacing_inv = 1.0 / box->spacing;
    for (int d = 0; d < 3; ++d) s->npm1[d] = box->npoints[d] - 1;
    const size_t P = (size_t)box->npoints[0] * box->npoints[1] * box->npoints[2];
    int all[PXD_NUM_VDW_TYPES];
    int nt = 0;
    if (n_types < 0) {
        for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) all[nt++] = t;
    } else {
        for (int t = 0; t < n_types; ++t) {
            int dup = 0;
            for (int u = 0; u < nt; ++u) dup |= (all[u] == types[t]);
            if (!dup) all[nt++] = types[t];
        }
    }
    s->maps[PXD_NUM_VDW_TYPES] = (double*)calloc(P * 4, sizeof(double));
    for (int t = 0; t < nt; ++t) s->maps[all[t]] = (double*)calloc(P * 4, sizeof(double));
    const int ni = box->npoints[0];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > ni) nthreads = ni;
    pthread_t* th = (pthread_t*)malloc((size_t)nthreads * sizeof(pthread_t));
    grid_job* jobs = (grid_job*)malloc((size_t)nthreads * sizeof(grid_job));
    const int len = (ni + nthreads - 1) / nthreads;
    for (int w = 0; w < nthreads; ++w) {
        jobs[w].s = s;
        jobs[w].types = all;
        jobs[w].n_types = nt;
        jobs[w].i0 = w * len < ni ? w * len : ni;
        jobs[w].i1 = (w + 1) * len < ni ? (w + 1) * len : ni;
        pthread_create(&th[w], NULL, grid_worker, &jobs[w]);
    }
    for (int w = 0; w < nthreads; ++w) pthread_join(th[w], NULL);
    free(th);
    free(jobs);
    s->has_grid = 1;
    return 0;
}

void po_set_slope(po_system* s, double slope) { s->slope = slope; }

void po_drop_grid(po_system* s) {
    for (int m = 0; m <= PXD_NUM_VDW_TYPES; ++m) {
        free(s->maps[m]);
        s->maps[m] = NULL;
    }
    s->has_grid = 0;
}

int po_grid_copy(const po_system* s, int map, double* out) {
    if (map < 0 || map > PXD_NUM_VDW_TYPES || !s->maps[map]) return -1;
    const size_t P = (size_t)s->box.npoints[0] * s->box.npoints[1] * s->box.npoints[2];
    memcpy(out, s->maps[map], P * 4 * sizeof(double));
    return 0;
}

static inline size_t grid_offset(const po_system* s, int i, int j, int k) {
    return ((size_t)i * s->box.npoints[1] + j) * s->box.npoints[2] + k;
}

/* Trilinear blend of the stored {E, grad} records (grid.cpp:273-303). */
static double trilinear(const double* m, const size_t* pidx, const double* w, double* grad) {
    double acc[4] = {0, 0, 0, 0};
    for (int c = 0; c < 8; ++c) {
        const double* f = m + 4 * pidx[c];
        double v[4] = {f[0] * w[c], f[1] * w[c], f[2] * w[c], f[3] * w[c]};
        if (c == 0) {
            memcpy(acc, v, sizeof(acc));
        } else {
            acc[0] += v[0];
            acc[1] += v[1];
            acc[2] += v[2];
            acc[3] += v[3];
        }
    }
    grad[0] = acc[1];
    grad[1] = acc[2];
    grad[2] = acc[3];
    return acc[0];
}

/* receptor_cache::get (grid.cpp:197-262). Returns 1 when the atom is inside. */
int po_grid_get(const po_system* s, int type, double q, const double* xyz, double* energy,
                double* grad) {
    double flb[3], gtmp[3], penalty = 0.0;
    int lo[3], hi[3];
    v_sub(xyz, s->box.init_xyz, flb);
    v_scalei(flb, s->spacing_inv);
    for (int d = 0; d < 3; ++d) {
        if (flb[d] < 0.0) {
            lo[d] = 0;
            gtmp[d] = -1.0;
            penalty -= flb[d];
            flb[d] = 0.0;
        } else if (flb[d] < s->npm1[d]) {
            lo[d] = (int)flb[d];
            gtmp[d] = 0.0;
        } else {
            lo[d] = s->npm1[d] - 1;
            gtmp[d] = 1.0;
            penalty += flb[d] - s->npm1[d];
            flb[d] = s->npm1[d];
        }
        hi[d] = lo[d] + 1;
    }
    size_t pidx[8];
    pidx[0] = grid_offset(s, lo[0], lo[1], lo[2]);
    pidx[1] = grid_offset(s, hi[0], lo[1], lo[2]);
    pidx[2] = grid_offset(s, lo[0], hi[1], lo[2]);
    pidx[3] = grid_offset(s, hi[0], hi[1], lo[2]);
    pidx[4] = grid_offset(s, lo[0], lo[1], hi[2]);
    pidx[5] = grid_offset(s, hi[0], lo[1], hi[2]);
    pidx[6] = grid_offset(s, lo[0], hi[1], hi[2]);
    pidx[7] = grid_offset(s, hi[0], hi[1], hi[2]);
    const double x = flb[0] - lo[0], y = flb[1] - lo[1], z = flb[2] - lo[2];
    const double mx = 1.0 - x, my = 1.0 - y, mz = 1.0 - z;
    const double w[8] = {mx * my * mz, x * my * mz, mx * y * mz, x * y * mz,
                         mx * my * z,  x * my * z,  mx * y * z,  x * y * z};
    int hit = 1;
    if (penalty > 0.0) {
        *energy += penalty * s->box.spacing * s->slope;
        v_scalei(gtmp, s->slope);
        v_addi(grad, gtmp);
        hit = 0;
    }
    *energy += trilinear(s->maps[PXD_NUM_VDW_TYPES], pidx, w, gtmp) * q;
    if (hit) {
        v_scalei(gtmp, q);
        v_addi(grad, gtmp);
    }
    *energy += trilinear(s->maps[type], pidx, w, gtmp);
    if (hit) v_addi(grad, gtmp);
    return hit;
}

/* ------------------------------------------- interaction.cpp:202-350 objective */
typedef struct {
    double* rec_xyz;  /* [n_rec][3] current receptor coordinates */
    double* rec_grad; /* [n_rec][3] */
    double* jac;      /* [n_mov][3] dR/dtheta . (x0 - origin) */
} po_work;

static void work_init(const po_system* s, po_work* w) {
    const size_t n = (size_t)(s->n_rec ? s->n_rec : 1);
    w->rec_xyz = (double*)malloc(n * 3 * sizeof(double));
    memcpy(w->rec_xyz, s->rec_xyz0, (size_t)s->n_rec * 3 * sizeof(double));
    w->rec_grad = (double*)malloc(n * 3 * sizeof(double));
    w->jac = (double*)malloc((size_t)(s->n_mov + 1) * 3 * sizeof(double));
}

static void work_free(po_work* w) {
    free(w->rec_xyz);
    free(w->rec_grad);
    free(w->jac);
}

static double score_grad_work(const po_system* s, po_work* w, const double* tors,
                              const double* lig_xyz, double* tgrad, double* lgrad) {
    /* receptor_torsion2xyz (interaction.cpp:316-336) */
    int off = 0;
    for (int r = 0; r < s->n_rotors; ++r) {
        double rot[9], jr[9], tmp[3];
        po_rotation_axis_angle(s->rotor_axis + 3 * r, tors[r], rot, jr);
        for (int k = s->mov_offsets[r]; k < s->mov_offsets[r + 1]; ++k) {
            const int j = s->mov_atoms[k];
            v_sub(s->rec_xyz0 + 3 * j, s->rotor_origin + 3 * r, tmp);
            m_apply(rot, tmp, w->rec_xyz + 3 * j);
            v_addi(w->rec_xyz + 3 * j, s->rotor_origin + 3 * r);
            m_apply(jr, tmp, w->jac + 3 * off);
            ++off;
        }
    }
    memset(w->rec_grad, 0, (size_t)s->n_rec * 3 * sizeof(double));
    memset(lgrad, 0, (size_t)s->n_lig * 3 * sizeof(double));
    double energy = 0.0;
    energy += po_intra_energy(4, &s->rec.t, w->rec_xyz, w->rec_grad);
    energy += po_intra_energy(4, &s->lig.t, lig_xyz, lgrad);
    /* inter_molecular_interactions::put_gradients (interaction.cpp:202-257) */
    double inter = 0.0;
    for (int i = 0; i < s->n_lig; ++i) {
        const double qi = s->lig.t.charge[i];
        const int ty = s->lig_type[i];
        const double si = PXD_VDW_SIGMA[ty], ei = PXD_VDW_EPSILON[ty];
        const int* list = s->has_grid ? s->excl_list : NULL;
        const int nlist = s->has_grid ? s->n_excl : s->n_rec;
        if (s->has_grid) po_grid_get(s, ty, qi, lig_xyz + 3 * i, &inter, lgrad + 3 * i);
        for (int k = 0; k < nlist; ++k) {
            const int j = list ? list[k] : k;
            double rij[3];
            v_sub(w->rec_xyz + 3 * j, lig_xyz + 3 * i, rij);
            const double d = v_norm(rij);
            inter += coul_pair(qi, s->rec.t.charge[j], rij, d, 1.0, lgrad + 3 * i, w->rec_grad + 3 * j);
            inter += vdw_pair(si, ei, s->rec.t.sigma[j], s->rec.t.epsilon[j], rij, d, 1.0,
                              lgrad + 3 * i, w->rec_grad + 3 * j);
        }
    }
    energy += inter;
    /* receptor_xyz2torsion (interaction.cpp:338-350) */
    off = 0;
    for (int r = 0; r < s->n_rotors; ++r) {
        tgrad[r] = 0.0;
        for (int k = s->mov_offsets[r]; k < s->mov_offsets[r + 1]; ++k) {
            tgrad[r] += v_dot(w->jac + 3 * off, w->rec_grad + 3 * s->mov_atoms[k]);
            ++off;
        }
    }
    return energy;
}

double po_score_grad(po_system* s, const double* tors, const double* lig_xyz, double* tgrad,
                     double* lgrad) {
    po_work w;
    work_init(s, &w);
    const double e = score_grad_work(s, &w, tors, lig_xyz, tgrad, lgrad);
    work_free(&w);
    return e;
}

/* ----------------------------------------------- L-BFGS (optimizer.cpp:56-560) */
typedef struct {
    const po_system* s;
    po_work* w;
    int D, n3, nt;
    const double* x0;  /* start [3N | T] flat */
    double* xt;        /* trial */
    double* tgrad;
    int32_t* nevals;
} closure_t;

static inline double vec_absmax(const double* a, int n) {
    double v = 0.0;
    for (int i = 0; i < n; ++i) {
        const double t = fabs(a[i]);
        if (t > v) v = t;
    }
    return v;
}
static inline double vec_abssum(const double* a, int n) {
    double v = 0.0;
    for (int i = 0; i < n; ++i) v += fabs(a[i]);
    return v;
}
static inline double vec_dot(const double* a, const double* b, int n) {
    double v = 0.0;
    for (int i = 0; i < n; ++i) v += a[i] * b[i];
    return v;
}

/* obj_func_closure::evaluate_direction (optimizer.cpp:155-167): f and flat gradient
 * at x0 + t * d, with the flat layout [ligand xyz | receptor torsions]. */
static double eval_dir(closure_t* c, double t, const double* d, double* g) {
    for (int i = 0; i < c->D; ++i) c->xt[i] = c->x0[i] + d[i] * t;
    const double e = score_grad_work(c->s, c->w, c->xt + c->n3, c->xt, c->tgrad, g);
    memcpy(g + c->n3, c->tgrad, (size_t)c->nt * sizeof(double));
    ++*c->nevals;
    return e;
}

/* model.put_gradients at the current x (optimizer.cpp:434-436, 554-558) */
static double eval_at_x(closure_t* c, double* g) {
    const double e = score_grad_work(c->s, c->w, c->x0 + c->n3, c->x0, c->tgrad, g);
    memcpy(g + c->n3, c->tgrad, (size_t)c->nt * sizeof(double));
    ++*c->nevals;
    return e;
}

/* cubic_interpolate (optimizer.cpp:205-233) */
static double cubic_interpolate(double x1, double f1, double g1, double x2, double f2, double g2,
                                double lo, double hi) {
    double d1 = g1 + g2 - 3.0 * (f1 - f2) / (x1 - x2);
    const double d2sq = d1 * d1 - g1 * g2;
    if (d2sq >= 0.0) {
        const double d2 = sqrt(d2sq);
        if (x1 <= x2)
            d1 = x2 - (x2 - x1) * ((g2 + d2 - d1) / (g2 - g1 + 2.0 * d2));
        else
            d1 = x1 - (x1 - x2) * ((g1 + d2 - d1) / (g1 - g2 + 2.0 * d2));
        const double m = d1 > lo ? d1 : lo;
        return m < hi ? m : hi;
    }
    return (lo + hi) / 2.0;
}

/* strong_wolfe (optimizer.cpp:235-427). g holds the current gradient on entry and the
 * accepted one on exit; bufs provides 4 scratch gradient vectors. */
static void strong_wolfe(closure_t* c, const pxd_lbfgs_params* p, double* t_io, const double* d,
                         double* f_io, double* g, double gtd, double** bufs) {
    const int D = c->D;
    double t = *t_io, f = *f_io;
    double* g_new = bufs[0];
    double* g_prev = bufs[1];
    double* bg[2] = {bufs[2], bufs[3]};
    double br[2] = {0, 0}, bf[2] = {0, 0}, bgtd[2] = {0, 0};
    double f_new = eval_dir(c, t, d, g_new);
    if (isnan(f_new)) {
        *f_io = f_new;
        return;
    }
    double gtd_new = vec_dot(g_new, d, D);
    if (fabs(gtd_new) > p->ls_gtd_threshold) {
        *f_io = f_new;
        memcpy(g, g_new, (size_t)D * sizeof(double));
        *t_io = t;
        return;
    }
    double t_prev = 0.0, f_prev = f, gtd_prev = gtd;
    memcpy(g_prev, g, (size_t)D * sizeof(double));
    int done = 0, ls_iter = 0;
    while (ls_iter < p->ls_max) {
        if ((f_new > f + p->ls_c1 * t * gtd) || (ls_iter > 1 && f_new >= f_prev)) {
            br[0] = t_prev; br[1] = t; bf[0] = f_prev; bf[1] = f_new;
            memcpy(bg[0], g_prev, (size_t)D * sizeof(double));
            memcpy(bg[1], g_new, (size_t)D * sizeof(double));
            bgtd[0] = gtd_prev; bgtd[1] = gtd_new;
            break;
        }
        if (fabs(gtd_new) <= -p->ls_c2 * gtd) {
            br[0] = t; bf[0] = f_new;
            memcpy(bg[0], g_new, (size_t)D * sizeof(double));
            done = 1;
            break;
        }
        if (gtd_new >= 0) {
            br[0] = t_prev; br[1] = t; bf[0] = f_prev; bf[1] = f_new;
            memcpy(bg[0], g_prev, (size_t)D * sizeof(double));
            memcpy(bg[1], g_new, (size_t)D * sizeof(double));
            bgtd[0] = gtd_prev; bgtd[1] = gtd_new;
            break;
        }
        const double min_step = t + 0.01 * (t - t_prev);
        const double max_step = t * 10.0;
        const double tmp = t;
        t = cubic_interpolate(t_prev, f_prev, gtd_prev, t, f_new, gtd_new, min_step, max_step);
        t_prev = tmp;
        f_prev = f_new;
        memcpy(g_prev, g_new, (size_t)D * sizeof(double));
        gtd_prev = gtd_new;
        f_new = eval_dir(c, t, d, g_new);
        gtd_new = vec_dot(g_new, d, D);
        ++ls_iter;
    }
    double d_norm = 0.0;
    if (ls_iter == p->ls_max) {
        br[0] = 0; br[1] = t; bf[0] = f; bf[1] = f_new;
        memcpy(bg[0], g, (size_t)D * sizeof(double));
        memcpy(bg[1], g_new, (size_t)D * sizeof(double));
    } else {
        d_norm = vec_absmax(d, D);
    }
    int insuf = 0, lo = 0, hi = 1;
    if (!done && bf[0] > bf[1]) {
        lo = 1;
        hi = 0;
    }
    while (!done && ls_iter < p->ls_max) {
        double min_step, max_step;
        if (br[0] > br[1]) {
            min_step = br[1];
            max_step = br[0];
        } else {
            min_step = br[0];
            max_step = br[1];
        }
        double eps = max_step - min_step;
        if (eps * d_norm < p->ls_tolerance_change) break;
        t = cubic_interpolate(br[0], bf[0], bgtd[0], br[1], bf[1], bgtd[1], min_step, max_step);
        eps *= 0.1;
        const double near = (max_step - t) < (t - min_step) ? (max_step - t) : (t - min_step);
        if (near < eps) {
            if (insuf || t >= max_step || t <= min_step) {
                if (fabs(t - max_step) < fabs(t - min_step))
                    t = max_step - eps;
                else
                    t = min_step + eps;
                insuf = 0;
            } else {
                insuf = 1;
            }
        } else {
            insuf = 0;
        }
        f_new = eval_dir(c, t, d, g_new);
        gtd_new = vec_dot(g_new, d, D);
        ++ls_iter;
        if (f_new > (f + p->ls_c1 * t * gtd) || f_new >= bf[lo]) {
            br[hi] = t;
            bf[hi] = f_new;
            memcpy(bg[hi], g_new, (size_t)D * sizeof(double));
            bgtd[hi] = gtd_new;
            if (bf[0] > bf[1]) {
                lo = 1;
                hi = 0;
            } else {
                lo = 0;
                hi = 1;
            }
        } else {
            if (fabs(gtd_new) <= -p->ls_c2 * gtd) {
                done = 1;
            } else if (gtd_new * (br[hi] - br[lo]) >= 0.0) {
                br[hi] = br[lo];
                bf[hi] = bf[lo];
                memcpy(bg[hi], bg[lo], (size_t)D * sizeof(double));
                bgtd[hi] = bgtd[lo];
            }
            br[lo] = t;
            bf[lo] = f_new;
            memcpy(bg[lo], g_new, (size_t)D * sizeof(double));
            bgtd[lo] = gtd_new;
        }
    }
    *t_io = br[lo];
    *f_io = bf[lo];
    memcpy(g, bg[lo], (size_t)D * sizeof(double));
}

static int lbfgs_work(const po_system* s, po_work* w, const pxd_lbfgs_params* p, double* tors,
                      double* lig_xyz, double* energy, int32_t* nevals) {
    const int n3 = 3 * s->n_lig, nt = s->n_rotors, D = n3 + nt;
    const int m = p->history;
    const int max_eval = p->max_eval > 0 ? p->max_eval : p->max_iter * 5 / 4;
    double* mem = (double*)calloc((size_t)D * (12 + 2 * (size_t)m) + 2 * (size_t)m + 8, sizeof(double));
    double* x = mem;           /* current [xyz | tors] */
    double* g = x + D;         /* flat gradient */
    double* gp = g + D;        /* previous flat gradient */
    double* d = gp + D;
    double* q = d + D;
    double* xt = q + D;
    double* tg = xt + D;
    double* bufs[4] = {tg + D, tg + 2 * D, tg + 3 * D, tg + 4 * D};
    double* S = tg + 5 * D;    /* [m][D] old_stps ring */
    double* Y = S + (size_t)m * D; /* [m][D] old_dirs ring */
    double* ro = Y + (size_t)m * D;
    double* al = ro + m;
    double* sv = al + m;       /* s = d * t */
    memcpy(x, lig_xyz, (size_t)n3 * sizeof(double));
    memcpy(x + n3, tors, (size_t)nt * sizeof(double));
    closure_t c = {s, w, D, n3, nt, x, xt, tg, nevals};
    *nevals = 0;
    /* initial f(x), df/dx */
    double loss = eval_at_x(&c, g);
    *energy = loss;
    int status = PXD_POSE_NOT_CONVERGED;
    if (vec_absmax(g, D) < p->tolerance_grad) {
        free(mem);
        return PXD_POSE_CONVERGED;
    }
    int head = 0, count = 0; /* ring buffer of the history deque */
    double H_diag = 1.0, t = 0.0, prev_loss;
    int n_iter = 0, updated = 0, high_change = 0;
    while (n_iter < p->max_iter && *nevals < max_eval) {
        ++n_iter;
        if (n_iter > 1) {
            for (int i = 0; i < D; ++i) q[i] = g[i] - gp[i]; /* y */
            high_change = vec_absmax(q, D) > p->reset_threshold;
        }
        if (n_iter == 1 || high_change) {
            for (int i = 0; i < D; ++i) d[i] = -g[i];
            head = count = 0;
            H_diag = 1.0;
        } else {
            double* y = q;
            for (int i = 0; i < D; ++i) sv[i] = d[i] * t;
            const double ys = vec_dot(y, sv, D);
            if (ys > 1e-10) {
                int slot;
                if (count == m) {
                    slot = head;
                    head = (head + 1) % m;
                } else {
                    slot = (head + count) % m;
                    ++count;
                }
                H_diag = ys / vec_dot(y, y, D);
                memcpy(Y + (size_t)slot * D, y, (size_t)D * sizeof(double));
                memcpy(S + (size_t)slot * D, sv, (size_t)D * sizeof(double));
                ro[slot] = 1.0 / ys;
            }
            for (int i = 0; i < D; ++i) q[i] = -g[i];
            for (int k = count - 1; k > -1; --k) {
                const int slot = (head + k) % m;
                al[k] = vec_dot(S + (size_t)slot * D, q, D) * ro[slot];
                const double* yy = Y + (size_t)slot * D;
                for (int i = 0; i < D; ++i) q[i] += yy[i] * (-al[k]);
            }
            for (int i = 0; i < D; ++i) d[i] = q[i] * H_diag;
            for (int k = 0; k < count; ++k) {
                const int slot = (head + k) % m;
                const double be = vec_dot(Y + (size_t)slot * D, d, D) * ro[slot];
                const double* ss = S + (size_t)slot * D;
                for (int i = 0; i < D; ++i) d[i] += ss[i] * (al[k] - be);
            }
        }
        memcpy(gp, g, (size_t)D * sizeof(double));
        prev_loss = loss;
        if (n_iter == 1 || high_change) {
            const double inv = 1.0 / vec_abssum(g, D);
            t = (1.0 < inv ? 1.0 : inv) * p->lr * 0.1;
        } else {
            t = p->lr;
        }
        const double gtd = vec_dot(g, d, D);
        if (gtd > -p->tolerance_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        strong_wolfe(&c, p, &t, d, &loss, g, gtd, bufs);
        if (isnan(loss)) {
            status = PXD_POSE_NAN;
            break;
        }
        for (int i = 0; i < D; ++i) x[i] += d[i] * t;
        updated = 1;
        if (vec_absmax(g, D) <= p->tolerance_grad) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        double smax = 0.0;
        for (int i = 0; i < D; ++i) {
            const double v = fabs(d[i] * t);
            if (v > smax) smax = v;
        }
        if (smax <= p->tolerance_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        if (fabs(loss - prev_loss) < p->tolerance_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
    }
    if (updated) {
        *energy = eval_at_x(&c, bufs[0]);
    }
    memcpy(lig_xyz, x, (size_t)n3 * sizeof(double));
    memcpy(tors, x + n3, (size_t)nt * sizeof(double));
    free(mem);
    return status;
}

int po_lbfgs(po_system* s, const pxd_lbfgs_params* p, double* tors, double* lig_xyz,
             double* energy, int32_t* nevals) {
    po_work w;
    work_init(s, &w);
    const int st = lbfgs_work(s, &w, p, tors, lig_xyz, energy, nevals);
    work_free(&w);
    return st;
}

typedef struct {
    po_system* s;
    const pxd_lbfgs_params* p;
    int n_poses;
    double *tors, *xyz, *energy;
    int32_t *nevals, *status;
    int next;
    pthread_mutex_t mtx;
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* b = (batch_job*)arg;
    po_work w;
    work_init(b->s, &w);
    const int n3 = 3 * b->s->n_lig, nt = b->s->n_rotors;
    while (1) {
        pthread_mutex_lock(&b->mtx);
        const int i = b->next++;
        pthread_mutex_unlock(&b->mtx);
        if (i >= b->n_poses) break;
        b->status[i] = lbfgs_work(b->s, &w, b->p, b->tors + (size_t)i * nt,
                                  b->xyz + (size_t)i * n3, b->energy + i, b->nevals + i);
    }
    work_free(&w);
    return NULL;
}

int po_lbfgs_batch(po_system* s, const pxd_lbfgs_params* p, int32_t n_poses, double* tors,
                   double* xyz, double* energy, int32_t* nevals, int32_t* status, int nthreads) {
    batch_job b = {s, p, n_poses, tors, xyz, energy, nevals, status, 0, PTHREAD_MUTEX_INITIALIZER};
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc((size_t)nthreads * sizeof(pthread_t));
    for (int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, batch_worker, &b);
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(th);
    return 0;
}

/* ------------------------------------------------------------ kinematics */
/* torsional_receptor::apply_parameters (data.cpp:366-385) */
void po_receptor_apply(const po_system* s, const double* tors, double* out) {
    memcpy(out, s->rec_xyz0, (size_t)s->n_rec * 3 * sizeof(double));
    for (int r = 0; r < s->n_rotors; ++r) {
        double rot[9], tmp[3];
        rotation_axis_angle(s->rotor_axis + 3 * r, tors[r], rot);
        for (int k = s->mov_offsets[r]; k < s->mov_offsets[r + 1]; ++k) {
            double* p = out + 3 * s->mov_atoms[k];
            v_sub(p, s->rotor_origin + 3 * r, tmp);
            m_apply(rot, tmp, p);
            v_addi(p, s->rotor_origin + 3 * r);
        }
    }
}

/* free_ligand::apply_parameters (data.cpp:592-641). The reference walks the fragment
 * tree recursively; the flat torsion list is in the same pre-order, so one pass over
 * it with per-fragment frames reproduces the same arithmetic:
 *   rel_i   = x_i - x_mine(f)           (post-order pass, data.cpp:544-559)
 *   fused_f = Rot(axis_f, theta_f) * fused_parent, fused_root = R
 *   world_i = fused_f * rel_i + origin_f, origin_f = world(x_mine(f)). */
void po_ligand_apply(const po_system* s, const double* xyz, const double* center,
                     const double* rot, const double* tors, double* out) {
    const int n = s->n_lig;
    double* c = (double*)malloc((size_t)n * 3 * sizeof(double));
    for (int p = 0; p < n; ++p) memcpy(c + 3 * p, xyz + 3 * s->perm[p], 3 * sizeof(double));
    const int F = s->n_frags;
    double* axes = (double*)calloc((size_t)F * 3, sizeof(double));
    double* fused = (double*)calloc((size_t)F * 9, sizeof(double));
    double* origin = (double*)calloc((size_t)F * 3, sizeof(double));
    int* is_root = (int*)calloc((size_t)F, sizeof(int));
    int* mine = (int*)malloc((size_t)F * sizeof(int));
    for (int r = 0; r < s->n_roots; ++r) is_root[s->roots[r]] = 1;
    for (int f = 0; f < F; ++f) mine[f] = -1;
    /* axes from the input pose (data.cpp:530-537) */
    for (int k = 0; k < s->n_tors; ++k) {
        const int f = s->tors_frag[k];
        mine[f] = s->tors_mine_atom[k];
        v_sub(c + 3 * s->tors_mine_atom[k], c + 3 * s->tors_parent_atom[k], axes + 3 * f);
        v_normalize(axes + 3 * f);
    }
    /* geometric centre over permuted order (data.h:101-106) */
    double old_center[3] = {0, 0, 0};
    for (int p = 0; p < n; ++p) v_addi(old_center, c + 3 * p);
    v_scalei(old_center, 1.0 / n);
    /* Relative coordinates (post_order_traverse, data.cpp:540-559). Every subtraction
     * there reads a mine atom that is still in input coordinates, so: first each
     * fragment's own atoms minus its mine atom, then each mine atom minus its parent's
     * mine atom (or the old centre under a root), children before parents. */
    for (int k = 0; k < s->n_tors; ++k) {
        const int f = s->tors_frag[k];
        for (int i = s->frag_start[f]; i < s->frag_end[f]; ++i)
            if (i != mine[f]) v_subi(c + 3 * i, c + 3 * mine[f]);
    }
    for (int k = s->n_tors - 1; k >= 0; --k) {
        const int f = s->tors_frag[k];
        const int pf = s->tors_parent[k];
        if (is_root[pf])
            v_subi(c + 3 * mine[f], old_center);
        else
            v_subi(c + 3 * mine[f], c + 3 * mine[pf]);
    }
    for (int r = 0; r < s->n_roots; ++r) {
        const int f = s->roots[r];
        for (int i = s->frag_start[f]; i < s->frag_end[f]; ++i) v_subi(c + 3 * i, old_center);
    }
    /* root frames (data.cpp:614-630) */
    double tmp[3];
    for (int r = 0; r < s->n_roots; ++r) {
        const int f = s->roots[r];
        memcpy(fused + 9 * f, rot, 9 * sizeof(double));
        memcpy(origin + 3 * f, center, 3 * sizeof(double));
        for (int i = s->frag_start[f]; i < s->frag_end[f]; ++i) {
            m_apply(rot, c + 3 * i, tmp);
            v_add(tmp, center, c + 3 * i);
        }
    }
    /* pre-order torsions (data.cpp:562-590, 632-638) */
    for (int k = 0; k < s->n_tors; ++k) {
        const int f = s->tors_frag[k];
        const int pf = s->tors_parent[k];
        /* the parent's frame moves this fragment's axis and mine atom */
        m_apply(fused + 9 * pf, axes + 3 * f, tmp);
        memcpy(axes + 3 * f, tmp, sizeof(tmp));
        m_apply(fused + 9 * pf, c + 3 * mine[f], tmp);
        v_add(tmp, origin + 3 * pf, c + 3 * mine[f]);
        double cur[9];
        rotation_axis_angle(axes + 3 * f, tors[k], cur);
        m_mul(cur, fused + 9 * pf, fused + 9 * f);
        memcpy(origin + 3 * f, c + 3 * mine[f], 3 * sizeof(double));
        for (int i = s->frag_start[f]; i < s->frag_end[f]; ++i) {
            if (i == mine[f]) continue;
            m_apply(fused + 9 * f, c + 3 * i, tmp);
            v_add(tmp, origin + 3 * f, c + 3 * i);
        }
    }
    for (int a = 0; a < n; ++a) memcpy(out + 3 * a, c + 3 * s->rev[a], 3 * sizeof(double));
    free(c);
    free(axes);
    free(fused);
    free(origin);
    free(is_root);
    free(mine);
}

/* ------------------------------------------------------- RNG (random.h:33-63) */
void po_rng_seed(po_rng* r, uint32_t seed) {
    r->mt[0] = seed;
    for (int i = 1; i < 624; ++i)
        r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->idx = 624;
}

/* MT19937 (Matsumoto & Nishimura 1998) */
uint32_t po_rng_next(po_rng* r) {
    if (r->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            const uint32_t y = (r->mt[i] & 0x80000000u) | (r->mt[(i + 1) % 624] & 0x7fffffffu);
            r->mt[i] = r->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        r->idx = 0;
    }
    uint32_t y = r->mt[r->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* std::uniform_int_distribution<int> over a 32-bit engine: libstdc++ reduces with
 * Lemire's multiply-and-reject method (arXiv:1805.10941). */
int po_rng_uniform_int(po_rng* r, int a, int b) {
    const uint32_t range = (uint32_t)b - (uint32_t)a + 1u;
    if (range == 0u) return (int)((uint32_t)a + po_rng_next(r));
    uint64_t prod = (uint64_t)po_rng_next(r) * range;
    uint32_t low = (uint32_t)prod;
    if (low < range) {
        const uint32_t threshold = (uint32_t)(-range) % range;
        while (low < threshold) {
            prod = (uint64_t)po_rng_next(r) * range;
            low = (uint32_t)prod;
        }
    }
    return (int)((uint32_t)a + (uint32_t)(prod >> 32));
}

/* std::generate_canonical<double, 53> over mt19937: two draws, (lo + hi * 2^32) / 2^64. */
static double canonical(po_rng* r) {
    double sum = (double)po_rng_next(r);
    sum += (double)po_rng_next(r) * 4294967296.0;
    double v = sum / 18446744073709551616.0;
    if (v >= 1.0) v = nextafter(1.0, 0.0);
    return v;
}

double po_rng_uniform_real(po_rng* r, double a, double b) { return canonical(r) * (b - a) + a; }
double po_rng_torsion(po_rng* r) { return canonical(r) * (kPi - -kPi) + -kPi; }

void po_rng_in_box(po_rng* r, const double* lo, const double* hi, double* out) {
    for (int d = 0; d < 3; ++d) out[d] = po_rng_uniform_real(r, lo[d], hi[d]);
}

/* random_orientation (random.cpp:29-40): uniform quaternion (Shoemake). */
void po_rng_orientation(po_rng* r, double* q) {
    const double two_pi = 2 * kPi;
    const double u1 = canonical(r) * (1.0 - 0.0) + 0.0;
    const double u2 = (canonical(r) * (1.0 - 0.0) + 0.0) * two_pi;
    const double u3 = (canonical(r) * (1.0 - 0.0) + 0.0) * two_pi;
    const double a = sqrt(1.0 - u1), b = sqrt(u1);
    q[0] = a * sin(u2);
    q[1] = a * cos(u2);
    q[2] = b * sin(u3);
    q[3] = b * cos(u3);
}

/* random_in_sphere (random.cpp:42-49): rejection in the cube [-1, 1)^3. */
void po_rng_in_sphere(po_rng* r, double* out) {
    while (1) {
        out[0] = canonical(r) * (1.0 - -1.0) + -1.0;
        out[1] = canonical(r) * (1.0 - -1.0) + -1.0;
        out[2] = canonical(r) * (1.0 - -1.0) + -1.0;
        if (v_sqsum(out) < 1.0) break;
    }
}

/* ============================================ empirical scores (scorer.cpp) */
static double ramp_down(double v, double lo, double hi) { /* math.h:196-206 */
    if (v < lo) return 1.0;
    if (v <= hi) return 1.0 - (v - lo) / (hi - lo);
    return 0.0;
}
static double ramp_down_c(double v, double c, double lo, double hi) { /* math.h:208-215 */
    return v < c ? ramp_down(c - v, lo, hi) : ramp_down(v - c, lo, hi);
}
static double clampd(double v, double lo, double hi) {
    const double m = v > lo ? v : lo;
    return m < hi ? m : hi;
}
static double dist(const double* a, const double* b) {
    double t = 0.0;
    t += (a[0] - b[0]) * (a[0] - b[0]);
    t += (a[1] - b[1]) * (a[1] - b[1]);
    t += (a[2] - b[2]) * (a[2] - b[2]);
    return sqrt(t);
}
static int ring_size(const int32_t* r) {
    int n = 0;
    while (n < 6 && r[n] >= 0) ++n;
    return n;
}
/* to_ring_centroid / to_ring_normal (scorer.cpp:128-172) */
static void ring_centroid(const double* x, const int32_t* r, double* c) {
    const int n = ring_size(r);
    c[0] = c[1] = c[2] = 0.0;
    for (int i = 0; i < n; ++i) v_addi(c, x + 3 * r[i]);
    c[0] /= n;
    c[1] /= n;
    c[2] /= n;
}
static void ring_normal(const double* x, const int32_t* r, double* nrm) {
    double e1[3], e2[3];
    v_sub(x + 3 * r[1], x + 3 * r[0], e1);
    v_sub(x + 3 * r[1], x + 3 * r[2], e2);
    v_cross(e1, e2, nrm);
    v_normalize(nrm);
}

typedef struct {
    int n;
    const double* xyz;
    const double* q;
    const double* sigma;   /* receptor: FF sigma; ligand: type table sigma */
    const double* eps;
    const int32_t* type;   /* ligand vdW types, NULL for the receptor */
    const pxd_score_lists* l;
} po_mol;

/* mm_interaction_vdw_energy::report (scorer.cpp:222-252) */
static double term_vdw(const pxd_sf_params* sf, const po_mol* R, const po_mol* L) {
    double e = 0.0;
    for (int i = 0; i < L->n; ++i) {
        const int t = L->type[i];
        const double s1 = PXD_VDW_SIGMA[t] * sf->vdw_sigma_scale[t];
        const double e1 = PXD_VDW_EPSILON[t] * sf->vdw_epsilon_scale[t];
        for (int j = 0; j < R->n; ++j) {
            const double d = dist(L->xyz + 3 * i, R->xyz + 3 * j);
            double fused = (s1 + R->sigma[j]) * 0.5;
            const double u6 = pow(safe_div(fused, d), 6.0);
            fused = sqrt(e1 * R->eps[j]) * 4.0;
            const double v = (u6 * u6 - u6) * fused;
            e += clampd(v, -sf->vdw_cutoff, sf->vdw_cutoff);
        }
    }
    return e * sf->vdw_scale;
}

/* mm_interaction_coulomb_energy::report (scorer.cpp:254-276) */
static double term_coulomb(const po_mol* R, const po_mol* L) {
    double e = 0.0;
    for (int i = 0; i < L->n; ++i)
        for (int j = 0; j < R->n; ++j)
            e += safe_div(L->q[i] * R->q[j], dist(L->xyz + 3 * i, R->xyz + 3 * j)) * kCoulomb;
    return e;
}

/* hydrophobic_energy::report (scorer.cpp:278-311) */
static double term_hydrophobic(const pxd_sf_params* sf, const po_mol* R, const po_mol* L) {
    double e = 0.0;
    for (int a = 0; a < L->l->n_hydrophobic; ++a) {
        const int i = L->l->hydrophobic[a];
        const double s1 = PXD_VDW_SIGMA[L->type[i]];
        for (int b = 0; b < R->l->n_hydrophobic; ++b) {
            const int j = R->l->hydrophobic[b];
            const double r1 = (s1 + R->sigma[j]) * sf->hydro_scale_factor + sf->hydro_dist_min;
            const double r2 = r1 + sf->hydro_dist_max;
            e -= ramp_down(dist(L->xyz + 3 * i, R->xyz + 3 * j), r1, r2);
        }
    }
    return e * sf->hydro_scale;
}

/* ionic_interaction_batch::calculate (scorer.cpp:337-368) */
static double ionic_batch(const double* cx, const int32_t* cat, int nc, const double* ax,
                          const int32_t* an, int na, const double* p) {
    double e = 0.0;
    for (int i = 0; i < nc; ++i)
        for (int j = 0; j < na; ++j) e -= ramp_down(dist(cx + 3 * cat[i], ax + 3 * an[j]), p[0], p[1]);
    return e;
}

static double term_ionic(const pxd_sf_params* sf, const po_mol* R, const po_mol* L) {
    double e = 0.0;
    e += sf->ionic_coef[0] * ionic_batch(L->xyz, L->l->cation, L->l->n_cation, R->xyz, R->l->anion,
                                         R->l->n_anion, sf->ionic[0]);
    e += sf->ionic_coef[1] * ionic_batch(R->xyz, R->l->cation, R->l->n_cation, L->xyz, L->l->anion,
                                         L->l->n_anion, sf->ionic[1]);
    return e;
}

/* cation_pi_interaction_batch::calculate (scorer.cpp:426-462) */
static double picat_batch(const double* cx, const int32_t* cat, int nc, const double* rx,
                          const int32_t* rings, int nr, const double* p) {
    double e = 0.0;
    for (int r = 0; r < nr; ++r) {
        double c[3];
        ring_centroid(rx, rings + 6 * r, c);
        for (int j = 0; j < nc; ++j) e -= ramp_down(dist(c, cx + 3 * cat[j]), p[0], p[1]);
    }
    return e;
}

static double term_picat(const pxd_sf_params* sf, const po_mol* R, const po_mol* L) {
    double e = 0.0;
    e += sf->picat_coef[0] * picat_batch(L->xyz, L->l->cation, L->l->n_cation, R->xyz, R->l->ring5,
                                         R->l->n_ring5, sf->picat[0]);
    e += sf->picat_coef[1] * picat_batch(L->xyz, L->l->cation, L->l->n_cation, R->xyz, R->l->ring6,
                                         R->l->n_ring6, sf->picat[1]);
    e += sf->picat_coef[2] * picat_batch(R->xyz, R->l->cation, R->l->n_cation, L->xyz, L->l->ring5,
                                         L->l->n_ring5, sf->picat[2]);
    e += sf->picat_coef[3] * picat_batch(R->xyz, R->l->cation, R->l->n_cation, L->xyz, L->l->ring6,
                                         L->l->n_ring6, sf->picat[3]);
    return e;
}

/* get_projected_centroid_distance / get_sigma_distance (scorer.cpp:615-636) */
static double projected(const double* n1, const double* c1, const double* c2) {
    double t[3];
    v_sub(c2, c1, t);
    const double dp = v_dot(n1, t);
    return sqrt(v_sqsum(t) - dp * dp);
}

/* pi_stacking_batch::calculate (scorer.cpp:698-724); p: dmin dmax amin amax smin smax */
static double stack_batch(const double* rx, const int32_t* rr, int nrr, const double* lx,
                          const int32_t* lr, int nlr, const double* p, double center) {
    double e = 0.0;
    for (int i = 0; i < nrr; ++i) {
        double rc[3], rn[3];
        ring_centroid(rx, rr + 6 * i, rc);
        ring_normal(rx, rr + 6 * i, rn);
        for (int j = 0; j < nlr; ++j) {
            double lc[3], ln[3];
            ring_centroid(lx, lr + 6 * j, lc);
            ring_normal(lx, lr + 6 * j, ln);
            double d = dist(rc, lc);
            if (d > p[1]) continue;
            d = ramp_down(d, p[0], p[1]);
            const double s1 = projected(rn, rc, lc), s2 = projected(ln, lc, rc);
            double sg = s1 < s2 ? s1 : s2;
            if (sg > p[5]) continue;
            sg = ramp_down(sg, p[4], p[5]);
            double th = acos(clampd(v_dot(rn, ln), -1.0, 1.0)) / kPi * 180.0;
            th = th < 180.0 - th ? th : 180.0 - th;
            th = ramp_down_c(th, center, p[2], p[3]);
            e -= d * sg * th;
        }
    }
    return e;
}

static double term_stack(const pxd_sf_params* sf, int which, const po_mol* R, const po_mol* L) {
    const double center = which == 0 ? 0.0 : 90.0;
    const double* c = sf->stack_coef[which];
    double e = 0.0;
    e += c[0] * stack_batch(R->xyz, R->l->ring5, R->l->n_ring5, L->xyz, L->l->ring5, L->l->n_ring5,
                            sf->stack[which][0], center);
    e += c[1] * stack_batch(R->xyz, R->l->ring6, R->l->n_ring6, L->xyz, L->l->ring5, L->l->n_ring5,
                            sf->stack[which][1], center);
    e += c[2] * stack_batch(R->xyz, R->l->ring5, R->l->n_ring5, L->xyz, L->l->ring6, L->l->n_ring6,
                            sf->stack[which][2], center);
    e += c[3] * stack_batch(R->xyz, R->l->ring6, R->l->n_ring6, L->xyz, L->l->ring6, L->l->n_ring6,
                            sf->stack[which][3], center);
    return e;
}

/* hbond_interactions_ga_tuning_param::calculate (scorer.cpp:546-577);
 * p: dist_min dist_max angle_min angle_max dist_center angle_center */
static double hbond_batch(const double* dx, const int32_t* don, int nd, const double* ax,
                          const int32_t* acc, int na, const double* p) {
    double e = 0.0;
    for (int i = 0; i < nd; ++i) {
        const double* dpos = dx + 3 * don[2 * i];
        const double* hpos = dx + 3 * don[2 * i + 1];
        for (int j = 0; j < na; ++j) {
            const double* apos = ax + 3 * acc[j];
            const double dd = ramp_down_c(dist(hpos, apos), p[4], p[0], p[1]);
            if (dd < EPS) continue;
            double h2d[3], h2a[3];
            v_sub(dpos, hpos, h2d);
            v_sub(apos, hpos, h2a);
            const double dp = clampd(safe_div(v_dot(h2d, h2a), v_norm(h2d) * v_norm(h2a)), -1.0, 1.0);
            const double ang = acos(dp) / kPi * 180.0;
            e -= dd * ramp_down_c(ang, p[5], p[2], p[3]);
        }
    }
    return e;
}

static double term_hbond(const pxd_sf_params* sf, const po_mol* R, const po_mol* L) {
    const pxd_score_lists *rl = R->l, *ll = L->l;
    const double* c = sf->hbond_coef;
    double e = 0.0;
    e += c[0] * hbond_batch(L->xyz, ll->don_charged, ll->n_don_charged, R->xyz, rl->acc_charged, rl->n_acc_charged, sf->hbond[0]);
    e += c[1] * hbond_batch(L->xyz, ll->don_charged, ll->n_don_charged, R->xyz, rl->acc_neutral, rl->n_acc_neutral, sf->hbond[1]);
    e += c[2] * hbond_batch(L->xyz, ll->don_neutral, ll->n_don_neutral, R->xyz, rl->acc_charged, rl->n_acc_charged, sf->hbond[2]);
    e += c[3] * hbond_batch(L->xyz, ll->don_neutral, ll->n_don_neutral, R->xyz, rl->acc_neutral, rl->n_acc_neutral, sf->hbond[3]);
    e += c[4] * hbond_batch(R->xyz, rl->don_charged, rl->n_don_charged, L->xyz, ll->acc_charged, ll->n_acc_charged, sf->hbond[4]);
    e += c[5] * hbond_batch(R->xyz, rl->don_charged, rl->n_don_charged, L->xyz, ll->acc_neutral, ll->n_acc_neutral, sf->hbond[5]);
    e += c[6] * hbond_batch(R->xyz, rl->don_neutral, rl->n_don_neutral, L->xyz, ll->acc_charged, ll->n_acc_charged, sf->hbond[6]);
    e += c[7] * hbond_batch(R->xyz, rl->don_neutral, rl->n_don_neutral, L->xyz, ll->acc_neutral, ll->n_acc_neutral, sf->hbond[7]);
    return e * sf->hbond_scale;
}

/* torsion_strain_penalty_scorer::report (scorer.cpp:579-613) */
double po_torsion_strain(const pxd_score_lists* l, const double* x) {
    static const double per[4] = {1.0, 2.0, 3.0, 4.0};
    static const double ph[4] = {0.0, 3.141592653589793, 0.0, 3.141592653589793};
    double score = 0.0;
    for (int e = 0; e < l->n_tstrain; ++e) {
        const double* co = l->tstrain_coefs + 4 * e;
        double tmp = 0.0;
        int j = 0;
        for (int q = l->tstrain_offsets[e]; q < l->tstrain_offsets[e + 1]; ++q, ++j) {
            const int32_t* a = l->tstrain_quads + 4 * q;
            if (a[0] == a[1]) break;
            const double th = po_dihedral(x + 3 * a[0], x + 3 * a[1], x + 3 * a[2], x + 3 * a[3]);
            tmp += (1 + cos(th * per[0] - ph[0])) * co[0] + (1 + cos(th * per[1] - ph[1])) * co[1] +
                   (1 + cos(th * per[2] - ph[2])) * co[2] + (1 + cos(th * per[3] - ph[3])) * co[3];
        }
        if (j > 0) score += tmp / j;
    }
    return score;
}

/* GBSA (scorer.cpp:737-866): radii and screens by element, Born radii, GB + SA. */
static const double kRadius[18] = {1.5, 1.2, 1.5, 1.5, 1.5, 1.5, 1.7, 1.55, 1.5,
                                   1.5, 1.5, 1.5, 1.5, 1.5, 2.1, 1.85, 1.8, 1.7};
static const double kScreen[17] = {0.8, 0.85, 0.8, 0.8, 0.8, 0.8, 0.72, 0.79, 0.85,
                                   0.88, 0.8, 0.8, 0.8, 0.8, 0.8, 0.86, 0.96};

static void gbsa_props(const po_mol* M, double* radii, double* screens) {
    const int n = M->n;
    for (int i = 0; i < n; ++i) radii[i] = -1.0;
    for (int b = 0; b < M->l->n_all_bonds; ++b) {
        const int i = M->l->all_bonds[2 * b], j = M->l->all_bonds[2 * b + 1];
        const int ea = M->l->atomic_numbers[i], eb = M->l->atomic_numbers[j];
        if (ea == 1 && eb == 7) radii[i] = 1.3;
        else if (ea == 7 && eb == 1) radii[j] = 1.3;
    }
    for (int i = 0; i < n; ++i) {
        const int e = M->l->atomic_numbers[i];
        if (radii[i] < 0.0) radii[i] = e <= 17 ? kRadius[e] : kRadius[0];
        screens[i] = e <= 16 ? kScreen[e] : kScreen[0];
    }
}

/* gbsa_total_energy::calculate (scorer.cpp:798-866) with the reference constants
 * (gbsa_total_energy constructor, scorer.h:400-408: solvent 78.5, solute 1, offset 0.09,
 * alpha 1, beta 0.8, gamma 4.85, probe 1.4, surface 0.0678584012906,
 * kappa 0.09293963686178248). */
static double gbsa_calc(int n, const double* x, const double* q, const double* radii,
                        const double* screens) {
    const double offset = 0.09, alpha = 1.0, beta = 0.8, gamma_ = 4.85;
    const double solute = 1.0, solvent = 78.5, kappa = 0.09293963686178248, probe = 1.4;
    const double surface = 0.0678584012906;
    double* orad = (double*)malloc((size_t)(n ? n : 1) * sizeof(double));
    double* sumI = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
    double* born = (double*)malloc((size_t)(n ? n : 1) * sizeof(double));
    for (int i = 0; i < n; ++i) orad[i] = radii[i] - offset;
    for (int i = 0; i < n; ++i) {
        const double sr = orad[i] * screens[i], sr2 = sr * sr;
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            const double r12 = dist(x + 3 * i, x + 3 * j);
            const double U = r12 + sr;
            if (U < orad[j]) continue;
            const double r12i = 1.0 / r12;
            double D = fabs(r12 - sr);
            const double L = orad[j] > D ? orad[j] : D;
            const double Ui = 1.0 / U, Li = 1.0 / L;
            D = 0.25 * (r12 - sr2 * r12i) * (Ui * Ui - Li * Li);
            D += (Li - Ui + 0.5 * log(L * Ui + EPS) * r12i);
            D *= 0.5;
            sumI[j] += D;
        }
    }
    for (int i = 0; i < n; ++i) {
        const double U = sumI[i] * orad[i];
        const double D = U * U;
        const double L = tanh(alpha * U - beta * D + gamma_ * U * D);
        born[i] = 1.0 / (1.0 / orad[i] - L / radii[i]);
    }
    double egb = 0.0;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            double f;
            if (i == j) {
                f = born[i];
            } else {
                double t = 0.0;
                t += (x[3 * i] - x[3 * j]) * (x[3 * i] - x[3 * j]);
                t += (x[3 * i + 1] - x[3 * j + 1]) * (x[3 * i + 1] - x[3 * j + 1]);
                t += (x[3 * i + 2] - x[3 * j + 2]) * (x[3 * i + 2] - x[3 * j + 2]);
                const double bp = born[i] * born[j];
                f = sqrt(t + bp * exp(-0.25 * t / bp) + EPS);
            }
            const double pref = 0.5 * kCoulomb * (1.0 / solute - exp(-kappa * f) / solvent);
            egb -= q[i] * q[j] / f * pref;
        }
    }
    double esa = 0.0;
    for (int i = 0; i < n; ++i)
        esa += (radii[i] + probe) * (radii[i] + probe) * pow(radii[i] / born[i], 6.0);
    free(orad);
    free(sumI);
    free(born);
    return egb + esa * surface;
}

/* gbsa_total_energy::summary: complex - ligand - receptor (scorer.cpp:755-796) */
static double term_gbsa(const po_mol* R, const po_mol* L, double* parts) {
    const int nr = R->n, nl = L->n, n = nr + nl;
    double* rr = (double*)malloc((size_t)(nr + 1) * sizeof(double));
    double* rs = (double*)malloc((size_t)(nr + 1) * sizeof(double));
    double* lr = (double*)malloc((size_t)(n + 1) * sizeof(double));
    double* ls = (double*)malloc((size_t)(n + 1) * sizeof(double));
    gbsa_props(R, rr, rs);
    const double e_pro = gbsa_calc(nr, R->xyz, R->q, rr, rs);
    gbsa_props(L, lr, ls);
    const double e_lig = gbsa_calc(nl, L->xyz, L->q, lr, ls);
    double* cx = (double*)malloc((size_t)(n + 1) * 3 * sizeof(double));
    double* cq = (double*)malloc((size_t)(n + 1) * sizeof(double));
    memcpy(cx, L->xyz, (size_t)nl * 3 * sizeof(double));
    memcpy(cx + 3 * nl, R->xyz, (size_t)nr * 3 * sizeof(double));
    memcpy(cq, L->q, (size_t)nl * sizeof(double));
    memcpy(cq + nl, R->q, (size_t)nr * sizeof(double));
    memcpy(lr + nl, rr, (size_t)nr * sizeof(double));
    memcpy(ls + nl, rs, (size_t)nr * sizeof(double));
    const double e_com = gbsa_calc(n, cx, cq, lr, ls);
    if (parts) {
        parts[0] = e_com;
        parts[1] = e_lig;
        parts[2] = e_pro;
    }
    free(rr);
    free(rs);
    free(lr);
    free(ls);
    free(cx);
    free(cq);
    return e_com - e_lig - e_pro;
}

/* root_scorer::combine over the active terms (scorer.cpp:53-126). terms[11] gets the
 * raw value of every active term (0 otherwise); returns sum(coef * term). */
double po_score(const pxd_sf_params* sf, int n_rec, const double* rec_xyz, const double* rec_q,
                const double* rec_sigma, const double* rec_eps, const pxd_score_lists* rec_l,
                int n_lig, const double* lig_xyz, const double* lig_q, const int32_t* lig_type,
                const pxd_score_lists* lig_l, double* terms) {
    po_mol R = {n_rec, rec_xyz, rec_q, rec_sigma, rec_eps, NULL, rec_l};
    po_mol L = {n_lig, lig_xyz, lig_q, NULL, NULL, lig_type, lig_l};
    double t[PXD_NUM_TERMS] = {0};
#define ACTIVE(k) (sf->coef[k] > 1e-5 || sf->coef[k] < -1e-5)
    if (ACTIVE(PXD_TERM_COULOMB)) t[PXD_TERM_COULOMB] = term_coulomb(&R, &L);
    if (ACTIVE(PXD_TERM_VDW)) t[PXD_TERM_VDW] = term_vdw(sf, &R, &L);
    if (ACTIVE(PXD_TERM_IONIC)) t[PXD_TERM_IONIC] = term_ionic(sf, &R, &L);
    if (ACTIVE(PXD_TERM_PI_CATION)) t[PXD_TERM_PI_CATION] = term_picat(sf, &R, &L);
    if (ACTIVE(PXD_TERM_F2F)) t[PXD_TERM_F2F] = term_stack(sf, 0, &R, &L);
    if (ACTIVE(PXD_TERM_E2F)) t[PXD_TERM_E2F] = term_stack(sf, 1, &R, &L);
    if (ACTIVE(PXD_TERM_HBOND)) t[PXD_TERM_HBOND] = term_hbond(sf, &R, &L);
    if (ACTIVE(PXD_TERM_HYDROPHOBIC)) t[PXD_TERM_HYDROPHOBIC] = term_hydrophobic(sf, &R, &L);
    if (ACTIVE(PXD_TERM_TSTRAIN)) t[PXD_TERM_TSTRAIN] = po_torsion_strain(lig_l, lig_xyz);
    if (ACTIVE(PXD_TERM_ROTATABLE)) t[PXD_TERM_ROTATABLE] = -1.0 / (2.620643 + lig_l->n_rotatable);
    if (ACTIVE(PXD_TERM_GBSA)) t[PXD_TERM_GBSA] = term_gbsa(&R, &L, NULL);
#undef ACTIVE
    double s = 0.0;
    for (int k = 0; k < PXD_NUM_TERMS; ++k) {
        if (terms) terms[k] = t[k];
        s += sf->coef[k] * t[k];
    }
    return s;
}

/* mm_interaction_vdw_energy::report alone: the randomize() clash check (searcher.cpp:76) */
double po_vdw_check(const pxd_sf_params* sf, int n_rec, const double* rec_xyz, const double* rec_sigma,
                    const double* rec_eps, int n_lig, const double* lig_xyz, const int32_t* lig_type) {
    po_mol R = {n_rec, rec_xyz, NULL, rec_sigma, rec_eps, NULL, NULL};
    po_mol L = {n_lig, lig_xyz, NULL, NULL, NULL, lig_type, NULL};
    return term_vdw(sf, &R, &L);
}

double po_gbsa_parts(int n_rec, const double* rec_xyz, const double* rec_q, const pxd_score_lists* rec_l,
                     int n_lig, const double* lig_xyz, const double* lig_q, const pxd_score_lists* lig_l,
                     double* parts) {
    po_mol R = {n_rec, rec_xyz, rec_q, NULL, NULL, NULL, rec_l};
    po_mol L = {n_lig, lig_xyz, lig_q, NULL, NULL, NULL, lig_l};
    return term_gbsa(&R, &L, parts);
}

/* ======================================= Monte-Carlo walker (searcher.cpp:46-223) */
static double geometric_center(const double* x, int n, double* c) {
    c[0] = c[1] = c[2] = 0.0;
    for (int i = 0; i < n; ++i) v_addi(c, x + 3 * i);
    v_scalei(c, 1.0 / n);
    return 0.0;
}

static int atom_in_box(const double* p, const double* lo, const double* hi) {
    return p[0] > lo[0] && p[0] < hi[0] && p[1] > lo[1] && p[1] < hi[1] && p[2] > lo[2] && p[2] < hi[2];
}

static int all_in_box(const double* x, int n, const double* lo, const double* hi) {
    for (int i = 0; i < n; ++i)
        if (!atom_in_box(x + 3 * i, lo, hi)) return 0;
    return 1;
}

typedef struct {
    const po_system* s;
    const pxd_sf_params* sf;
    const pxd_score_lists* rl;
    const pxd_score_lists* ll;
    const double* rec_q;
    const double* rec_sigma;
    const double* rec_eps;
} mc_env;

static double mc_pscore(const mc_env* e, const double* tors, const double* xyz, double* rec_buf) {
    po_receptor_apply(e->s, tors, rec_buf);
    return po_score(e->sf, e->s->n_rec, rec_buf, e->s->rec.t.charge, e->s->rec.t.sigma, e->s->rec.t.epsilon,
                    e->rl, e->s->n_lig, xyz, e->s->lig.t.charge, e->s->lig_type, e->ll, NULL);
}

/* randomize (searcher.cpp:46-87) */
static void mc_randomize(const mc_env* e, const double* start, int first_pose, const double* lo,
                         const double* hi, po_rng* rg, double* out) {
    const po_system* s = e->s;
    const int n = s->n_lig, T = s->n_tors;
    double center[3], q[4], R[9];
    double* tors = (double*)calloc((size_t)(T + 1), sizeof(double));
    int num = 0;
    while (1) {
        po_rng_in_box(rg, lo, hi, center);
        po_rng_orientation(rg, q);
        for (int i = 0; i < T; ++i)
            if (first_pose) tors[i] = po_rng_torsion(rg);
        po_rotation_quaternion(q, R);
        po_ligand_apply(s, start, center, R, tors, out);
        ++num;
        if (num < 2000 && !all_in_box(out, n, lo, hi)) continue;
        double c[3];
        geometric_center(out, n, c);
        if (!atom_in_box(c, lo, hi)) continue;
        if (num > 1999 || po_vdw_check(e->sf, s->n_rec, s->rec_xyz0, e->rec_sigma, e->rec_eps, n, out,
                                       s->lig_type) < 100.0)
            break;
    }
    free(tors);
}

/* mutate_inplace (searcher.cpp:189-223); returns 0 when the rotation was skipped */
static int mc_mutate(const po_system* s, po_rng* rg, double* xyz) {
    const int n = s->n_lig, T = s->n_tors;
    const int which = po_rng_uniform_int(rg, 0, T + 1);
    double center[3], delta[3];
    geometric_center(xyz, n, center);
    if (which == 0) {
        po_rng_in_sphere(rg, delta);
        v_scalei(delta, 2.0);
        v_addi(center, delta);
    }
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (which == 1) {
        double acc = 0.0;
        for (int i = 0; i < n; ++i) {
            double t = 0.0;
            t += (xyz[3 * i] - center[0]) * (xyz[3 * i] - center[0]);
            t += (xyz[3 * i + 1] - center[1]) * (xyz[3 * i + 1] - center[1]);
            t += (xyz[3 * i + 2] - center[2]) * (xyz[3 * i + 2] - center[2]);
            acc += t;
        }
        double gr = n > 0 ? sqrt(acc / n) : 0.0;
        if (gr < 1e-6) return 0;
        po_rng_in_sphere(rg, delta);
        v_scalei(delta, 2.0 / gr);
        gr = v_norm(delta);
        v_scalei(delta, 1.0 / gr);
        rotation_axis_angle(delta, gr, R);
    }
    double* tors = (double*)calloc((size_t)(T + 1), sizeof(double));
    if (which > 1) tors[which - 2] = po_rng_torsion(rg);
    double* tmp = (double*)malloc((size_t)n * 3 * sizeof(double));
    po_ligand_apply(s, xyz, center, R, tors, tmp);
    memcpy(xyz, tmp, (size_t)n * 3 * sizeof(double));
    free(tmp);
    free(tors);
    return 1;
}

typedef struct {
    double* xyz;
    double* tors;
    double energy, pscore;
    long nevals;
} mc_state;

static void mc_copy(mc_state* d, const mc_state* s, int n, int T) {
    memcpy(d->xyz, s->xyz, (size_t)n * 3 * sizeof(double));
    memcpy(d->tors, s->tors, (size_t)(T + 1) * sizeof(double));
    d->energy = s->energy;
    d->pscore = s->pscore;
    d->nevals = s->nevals;
}

/* One walker of monte_carlo_searcher::mutate_and_optimize (searcher.cpp:98-187).
 * start: the ligand pose the walker starts from; first_pose: 1 when that pose is the
 * file's first pose (then torsions are randomised as well). walker 0 only relaxes.
 * global_min: the shared pre-optimisation energy minimum when threshold > 0.
 * Returns 0 ok, 1 crashed (nevals set to 0), 2 relaxed start left the box. */
int po_mc_walker(po_system* s, const pxd_sf_params* sf, const pxd_score_lists* rl, const pxd_score_lists* ll,
                 const double* lo, const double* hi, uint32_t seed, int walker, const double* start,
                 int first_pose, int max_nsteps, int relax_nsteps, double threshold, double* global_min,
                 double* out_xyz, double* out_tors, double* out_energy, double* out_pscore, long* out_nevals) {
    const int n = s->n_lig, R = s->n_rotors;
    mc_env e = {s, sf, rl, ll, s->rec.t.charge, s->rec.t.sigma, s->rec.t.epsilon};
    po_rng rg;
    po_rng_seed(&rg, seed + (uint32_t)walker);
    double* rec_buf = (double*)malloc((size_t)(s->n_rec + 1) * 3 * sizeof(double));
    double* mem = (double*)calloc((size_t)3 * (3 * n + R + 1), sizeof(double));
    mc_state out = {mem, mem + 3 * n, 0, 0, 0};
    mc_state tmp = {mem + 3 * n + R + 1, mem + 6 * n + R + 1, 0, 0, 0};
    mc_state cdd = {mem + 6 * n + 2 * R + 2, mem + 9 * n + 2 * R + 2, 0, 0, 0};
    pxd_lbfgs_params full, fast;
    full.max_iter = 240; full.max_eval = 0; full.history = 100; full.ls_max = 25; full.lr = 1.0;
    full.tolerance_grad = 0.5; full.tolerance_change = 1e-4; full.ls_c1 = 1e-4; full.ls_c2 = 0.9;
    full.ls_tolerance_change = 1e-9; full.ls_gtd_threshold = 1e5; full.reset_threshold = 1e8;
    fast = full;
    fast.max_iter = relax_nsteps;
    po_work w;
    work_init(s, &w);
    int32_t nev = 0;
    if (walker == 0)
        memcpy(out.xyz, start, (size_t)n * 3 * sizeof(double));
    else
        mc_randomize(&e, start, first_pose, lo, hi, &rg, out.xyz);
    lbfgs_work(s, &w, &full, out.tors, out.xyz, &out.energy, &nev);
    out.nevals = nev;
    out.pscore = mc_pscore(&e, out.tors, out.xyz, rec_buf);
    int status = 0;
    if (walker != 0) {
        if (all_in_box(out.xyz, n, lo, hi)) {
            mc_copy(&tmp, &out, n, R);
            long total = out.nevals;
            for (int step = 0; step < max_nsteps; ++step) {
                mc_copy(&cdd, &tmp, n, R);
                mc_mutate(s, &rg, cdd.xyz);
                if (threshold > 0.0 && global_min) {
                    double tg[PXD_MAX_RECEPTOR_TORSIONS + 1];
                    double* lg = (double*)malloc((size_t)n * 3 * sizeof(double));
                    const double pre = score_grad_work(s, &w, cdd.tors, cdd.xyz, tg, lg);
                    free(lg);
                    if (pre < *global_min) *global_min = pre;
                    if (pre > *global_min + threshold) continue;
                }
                lbfgs_work(s, &w, &fast, cdd.tors, cdd.xyz, &cdd.energy, &nev);
                cdd.nevals = nev;
                total += cdd.nevals;
                cdd.pscore = mc_pscore(&e, cdd.tors, cdd.xyz, rec_buf);
                int accept = step == 0;
                if (!accept) {
                    if (cdd.pscore < tmp.pscore)
                        accept = 1;
                    else
                        accept = po_rng_uniform_real(&rg, 0.0, 1.0) < exp((tmp.pscore - cdd.pscore) / 1.2);
                }
                if (accept && all_in_box(cdd.xyz, n, lo, hi)) {
                    mc_copy(&tmp, &cdd, n, R);
                    if (tmp.pscore < out.pscore) {
                        lbfgs_work(s, &w, &full, tmp.tors, tmp.xyz, &tmp.energy, &nev);
                        tmp.nevals = nev;
                        total += tmp.nevals;
                        tmp.pscore = mc_pscore(&e, tmp.tors, tmp.xyz, rec_buf);
                        if (tmp.pscore < out.pscore) mc_copy(&out, &tmp, n, R);
                    }
                }
            }
            out.nevals = total;
        } else {
            int big = 0;
            for (int i = 0; i < 3 * n; ++i) big |= (out.xyz[i] > 1e8 || out.xyz[i] < -1e8);
            if (big) {
                out.nevals = 0;
                status = 1;
            } else {
                status = 2;
            }
        }
    }
    memcpy(out_xyz, out.xyz, (size_t)n * 3 * sizeof(double));
    memcpy(out_tors, out.tors, (size_t)R * sizeof(double));
    *out_energy = out.energy;
    *out_pscore = out.pscore;
    *out_nevals = out.nevals;
    work_free(&w);
    free(mem);
    free(rec_buf);
    return status;
}

/* The random start of walker `walker` alone (searcher.cpp:46-87): the pose randomize()
 * returns for the generator mt19937(seed + walker). */
void po_mc_randomize(po_system* s, const pxd_sf_params* sf, const double* lo, const double* hi,
                     uint32_t seed, int walker, const double* start, int first_pose, double* out) {
    mc_env e = {s, sf, NULL, NULL, s->rec.t.charge, s->rec.t.sigma, s->rec.t.epsilon};
    po_rng rg;
    po_rng_seed(&rg, seed + (uint32_t)walker);
    mc_randomize(&e, start, first_pose, lo, hi, &rg, out);
}

/* ============================== differentiable empirical score (no reference code) */
/* The weights / features / pair-table split of the empirical score and its analytic
 * adjoint, in FP64. The features are the unweighted sums of the leaf scorers above
 * (scorer.cpp:222-613); combining them with pxd_sf_weights(sf) and every term active
 * gives po_score. Gradients: ramps -1/(hi-lo) inside [lo, hi]; clamped LJ 0 beyond the
 * cut-off; acos' = -1/sqrt(1-c^2) inside the clamp; ring centroids share their gradient
 * equally, normals through n = (p1-p0) x (p1-p2) and its normalisation; dihedrals by
 * po_dihedral_and_gradient. */
static double ramp_down_d(double v, double lo, double hi) {
    return (v >= lo && v <= hi) ? -1.0 / (hi - lo) : 0.0;
}
static double ramp_c_vd(double v, double c, double lo, double hi, double* dv) {
    if (v < c) {
        *dv = -ramp_down_d(c - v, lo, hi);
        return ramp_down(c - v, lo, hi);
    }
    *dv = ramp_down_d(v - c, lo, hi);
    return ramp_down(v - c, lo, hi);
}
static void gacc(double* G, int i, const double* g, double s) {
    if (!G) return;
    G[3 * i] += s * g[0];
    G[3 * i + 1] += s * g[1];
    G[3 * i + 2] += s * g[2];
}
/* gradient on a ligand ring's centroid (gc) and unit normal (gn) onto its atoms */
static void ring_backward(const double* x, const int32_t* r, const double* gc, const double* gn, double* G) {
    if (!G) return;
    const int n = ring_size(r);
    for (int k = 0; k < n; ++k) gacc(G, r[k], gc, 1.0 / n);
    double a[3], b[3], nv[3], u[3], gnn[3], ga[3], gb[3];
    v_sub(x + 3 * r[1], x + 3 * r[0], a);
    v_sub(x + 3 * r[1], x + 3 * r[2], b);
    v_cross(a, b, nv);
    const double len = v_norm(nv);
    v_scale(nv, 1.0 / len, u);
    const double gu = v_dot(gn, u);
    for (int d = 0; d < 3; ++d) gnn[d] = (gn[d] - gu * u[d]) / len;
    v_cross(b, gnn, ga);
    v_cross(gnn, a, gb);
    gacc(G, r[0], ga, -1.0);
    gacc(G, r[1], ga, 1.0);
    gacc(G, r[1], gb, 1.0);
    gacc(G, r[2], gb, -1.0);
}
static int pair_class_d(int rec, int z) {
    if (z < 2) return -1;
    if (z == 6) return 0;
    if (z == 7) return 1;
    if (z == 8) return 2;
    if (rec) return 3;
    switch (z) {
        case 16: return 3;
        case 15: return 4;
        case 9: return 5;
        case 17: return 6;
        default: return 7;
    }
}

double po_combine_features(const double* w, const double* f) {
    double s = w[PXD_W_COEF + PXD_TERM_COULOMB] * f[0];
    s += w[PXD_W_COEF + PXD_TERM_VDW] * w[PXD_W_VDW_SCALE] * f[1];
    s += w[PXD_W_COEF + PXD_TERM_IONIC] * (w[PXD_W_IONIC] * f[2] + w[PXD_W_IONIC + 1] * f[3]);
    double t = 0.0;
    for (int k = 0; k < 4; ++k) t += w[PXD_W_PICAT + k] * f[4 + k];
    s += w[PXD_W_COEF + PXD_TERM_PI_CATION] * t;
    for (int q = 0; q < 2; ++q) {
        t = 0.0;
        for (int k = 0; k < 4; ++k) t += w[PXD_W_STACK + 4 * q + k] * f[8 + 4 * q + k];
        s += w[PXD_W_COEF + PXD_TERM_F2F + q] * t;
    }
    t = 0.0;
    for (int k = 0; k < 8; ++k) t += w[PXD_W_HBOND + k] * f[16 + k];
    s += w[PXD_W_COEF + PXD_TERM_HBOND] * w[PXD_W_HBOND_SCALE] * t;
    s += w[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] * w[PXD_W_HYDRO_SCALE] * f[24];
    s += w[PXD_W_COEF + PXD_TERM_TSTRAIN] * f[25];
    s += w[PXD_W_COEF + PXD_TERM_ROTATABLE] * f[26];
    return s + f[27];
}

void po_combine_grad(const double* w, const double* f, double g, double* dw) {
    double hb = 0.0, pc = 0.0, st[2] = {0.0, 0.0};
    for (int k = 0; k < 8; ++k) hb += w[PXD_W_HBOND + k] * f[16 + k];
    for (int k = 0; k < 4; ++k) pc += w[PXD_W_PICAT + k] * f[4 + k];
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 4; ++k) st[q] += w[PXD_W_STACK + 4 * q + k] * f[8 + 4 * q + k];
    double d[PXD_NUM_SF_WEIGHTS] = {0};
    d[PXD_W_COEF + PXD_TERM_COULOMB] = f[0];
    d[PXD_W_COEF + PXD_TERM_VDW] = w[PXD_W_VDW_SCALE] * f[1];
    d[PXD_W_COEF + PXD_TERM_IONIC] = w[PXD_W_IONIC] * f[2] + w[PXD_W_IONIC + 1] * f[3];
    d[PXD_W_COEF + PXD_TERM_PI_CATION] = pc;
    d[PXD_W_COEF + PXD_TERM_F2F] = st[0];
    d[PXD_W_COEF + PXD_TERM_E2F] = st[1];
    d[PXD_W_COEF + PXD_TERM_HBOND] = w[PXD_W_HBOND_SCALE] * hb;
    d[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] = w[PXD_W_HYDRO_SCALE] * f[24];
    d[PXD_W_COEF + PXD_TERM_TSTRAIN] = f[25];
    d[PXD_W_COEF + PXD_TERM_ROTATABLE] = f[26];
    d[PXD_W_VDW_SCALE] = w[PXD_W_COEF + PXD_TERM_VDW] * f[1];
    d[PXD_W_HYDRO_SCALE] = w[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] * f[24];
    d[PXD_W_HBOND_SCALE] = w[PXD_W_COEF + PXD_TERM_HBOND] * hb;
    for (int k = 0; k < 2; ++k) d[PXD_W_IONIC + k] = w[PXD_W_COEF + PXD_TERM_IONIC] * f[2 + k];
    for (int k = 0; k < 4; ++k) d[PXD_W_PICAT + k] = w[PXD_W_COEF + PXD_TERM_PI_CATION] * f[4 + k];
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 4; ++k) d[PXD_W_STACK + 4 * q + k] = w[PXD_W_COEF + PXD_TERM_F2F + q] * f[8 + 4 * q + k];
    for (int k = 0; k < 8; ++k) d[PXD_W_HBOND + k] = w[PXD_W_COEF + PXD_TERM_HBOND] * w[PXD_W_HBOND_SCALE] * f[16 + k];
    for (int k = 0; k < PXD_NUM_SF_WEIGHTS; ++k) dw[k] += g * d[k];
}

/* pi_stacking_batch::calculate for one ring pair; adds s * d(value) to glc / gln */
static double stack_pair_diff(const double* rc, const double* rn, const double* lc, const double* ln, const double* p,
                              double center, double s, double* glc, double* gln) {
    double t[3], t2[3];
    v_sub(lc, rc, t);
    const double dist = v_norm(t);
    if (dist > p[1]) return 0.0;
    const double D = ramp_down(dist, p[0], p[1]);
    const double dp1 = v_dot(rn, t);
    const double s1 = sqrt(v_sqsum(t) - dp1 * dp1);
    v_sub(rc, lc, t2);
    const double dp2 = v_dot(ln, t2);
    const double s2 = sqrt(v_sqsum(t2) - dp2 * dp2);
    const int first = s1 < s2;
    const double sg = first ? s1 : s2;
    if (sg > p[5]) return 0.0;
    const double SG = ramp_down(sg, p[4], p[5]);
    const double c = clampd(v_dot(rn, ln), -1.0, 1.0);
    double th = acos(c) / kPi * 180.0, sign = 1.0;
    if (180.0 - th < th) {
        th = 180.0 - th;
        sign = -1.0;
    }
    double dTH;
    const double TH = ramp_c_vd(th, center, p[2], p[3], &dTH);
    if (glc && s != 0.0) {
        const double dD = ramp_down_d(dist, p[0], p[1]), dSG = ramp_down_d(sg, p[4], p[5]);
        double g_lc[3] = {0, 0, 0}, g_ln[3] = {0, 0, 0};
        if (dD != 0.0 && dist > 0.0)
            for (int d = 0; d < 3; ++d) g_lc[d] += t[d] * dD * SG * TH / dist;
        if (dSG != 0.0 && sg > 0.0) {
            const double k = D * dSG * TH / sg;
            for (int d = 0; d < 3; ++d) {
                if (first) {
                    g_lc[d] += (t[d] - rn[d] * dp1) * k;
                } else {
                    g_lc[d] -= (t2[d] - ln[d] * dp2) * k;
                    g_ln[d] -= t2[d] * dp2 * k;
                }
            }
        }
        const double dot = v_dot(rn, ln);
        if (dTH != 0.0 && dot > -1.0 && dot < 1.0) {
            const double dth_dc = -(180.0 / kPi) / sqrt(1.0 - c * c);
            for (int d = 0; d < 3; ++d) g_ln[d] += rn[d] * D * SG * dTH * sign * dth_dc;
        }
        for (int d = 0; d < 3; ++d) {
            glc[d] -= s * g_lc[d];
            gln[d] -= s * g_ln[d];
        }
    }
    return -D * SG * TH;
}

/* hbond_interactions_ga_tuning_param::calculate for one pair; adds s * d(value) */
static double hbond_pair_diff(const double* dpos, const double* hpos, const double* apos, const double* p, double s,
                              double* gd, double* gh, double* ga) {
    double ha[3], u[3], v[3];
    v_sub(hpos, apos, ha);
    const double D = v_norm(ha);
    double ddd;
    const double dd = ramp_c_vd(D, p[4], p[0], p[1], &ddd);
    if (dd < EPS) return 0.0;
    v_sub(dpos, hpos, u);
    v_sub(apos, hpos, v);
    const double lu = v_norm(u), lv = v_norm(v), L = lu * lv + EPS, uv = v_dot(u, v);
    const double cr = uv / L;
    const double c = clampd(cr, -1.0, 1.0);
    const double ang = acos(c) / kPi * 180.0;
    double dAR;
    const double AR = ramp_c_vd(ang, p[5], p[2], p[3], &dAR);
    if (gh && s != 0.0) {
        if (ddd != 0.0 && D > 0.0)
            for (int d = 0; d < 3; ++d) {
                const double g = -s * ddd * AR / D * ha[d];
                gh[d] += g;
                ga[d] -= g;
            }
        if (dAR != 0.0 && cr > -1.0 && cr < 1.0 && lu > 0.0 && lv > 0.0) {
            const double k = -s * dd * dAR * (-(180.0 / kPi) / sqrt(1.0 - c * c));
            for (int d = 0; d < 3; ++d) {
                const double dcu = v[d] / L - u[d] * uv * lv / (lu * L * L);
                const double dcv = u[d] / L - v[d] * uv * lu / (lv * L * L);
                gd[d] += k * dcu;
                ga[d] += k * dcv;
                gh[d] -= k * (dcu + dcv);
            }
        }
    }
    return -dd * AR;
}

double po_score_diff(const pxd_sf_params* sf, int n_rec, const double* rec_xyz, const double* rec_q,
                     const double* rec_sigma, const double* rec_eps, const pxd_score_lists* rl, int n_lig,
                     const double* x, const double* lig_q, const int32_t* lig_type, const pxd_score_lists* ll,
                     const double* w, const double* table, double g, double* f, double* G, double* dw, double* dtab) {
    double fl[PXD_NUM_SCORE_FEATURES] = {0};
    const double s_coul = g * w[PXD_W_COEF + PXD_TERM_COULOMB] * kCoulomb;
    const double s_vdw = g * w[PXD_W_COEF + PXD_TERM_VDW] * w[PXD_W_VDW_SCALE];
    const int use_tab = table && rl->atomic_numbers && ll->atomic_numbers;
    /* Coulomb, clamped LJ (scorer.cpp:222-276) and the pair table */
    for (int i = 0; i < n_lig; ++i) {
        const int t = lig_type[i];
        const double s1 = PXD_VDW_SIGMA[t] * sf->vdw_sigma_scale[t];
        const double e1 = PXD_VDW_EPSILON[t] * sf->vdw_epsilon_scale[t];
        const int ci = use_tab ? pair_class_d(0, ll->atomic_numbers[i]) : -1;
        for (int j = 0; j < n_rec; ++j) {
            double dv[3];
            v_sub(x + 3 * i, rec_xyz + 3 * j, dv);
            const double d = v_norm(dv);
            const double rinv = 1.0 / (d + EPS);
            fl[0] += lig_q[i] * rec_q[j] * rinv * kCoulomb;
            const double u6 = pow((s1 + rec_sigma[j]) * 0.5 * rinv, 6.0);
            const double fused = sqrt(e1 * rec_eps[j]) * 4.0;
            const double v = (u6 * u6 - u6) * fused;
            fl[1] += clampd(v, -sf->vdw_cutoff, sf->vdw_cutoff);
            double de_dd = -s_coul * lig_q[i] * rec_q[j] * rinv * rinv;
            if (v <= sf->vdw_cutoff && v >= -sf->vdw_cutoff) de_dd -= s_vdw * fused * rinv * (12.0 * u6 * u6 - 6.0 * u6);
            const int cj = ci >= 0 ? pair_class_d(1, rl->atomic_numbers[j]) : -1;
            const double tt = d / PXD_PAIR_BIN_WIDTH;
            if (cj >= 0 && tt < PXD_PAIR_BINS - 1) {
                const int b = (int)tt;
                const double fr = tt - b;
                const int p = (4 * ci + cj) * PXD_PAIR_BINS + b;
                fl[27] += table[p] + fr * (table[p + 1] - table[p]);
                de_dd += g * (table[p + 1] - table[p]) / PXD_PAIR_BIN_WIDTH;
                if (dtab) {
                    dtab[p] += g * (1.0 - fr);
                    dtab[p + 1] += g * fr;
                }
            }
            if (d > 0.0) gacc(G, i, dv, de_dd / d);
        }
    }
    /* hydrophobic (scorer.cpp:278-311) */
    {
        const double sh = g * w[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] * w[PXD_W_HYDRO_SCALE];
        for (int a = 0; a < ll->n_hydrophobic; ++a) {
            const int i = ll->hydrophobic[a];
            const double s1 = PXD_VDW_SIGMA[lig_type[i]];
            for (int b = 0; b < rl->n_hydrophobic; ++b) {
                const int j = rl->hydrophobic[b];
                const double r1 = (s1 + rec_sigma[j]) * sf->hydro_scale_factor + sf->hydro_dist_min;
                const double r2 = r1 + sf->hydro_dist_max;
                double dv[3];
                v_sub(x + 3 * i, rec_xyz + 3 * j, dv);
                const double d = v_norm(dv);
                fl[24] -= ramp_down(d, r1, r2);
                if (d > 0.0) gacc(G, i, dv, -sh * ramp_down_d(d, r1, r2) / d);
            }
        }
    }
    /* ionic (scorer.cpp:313-368) */
    for (int k = 0; k < 2; ++k) {
        const double sk = g * w[PXD_W_COEF + PXD_TERM_IONIC] * w[PXD_W_IONIC + k];
        const int na = k == 0 ? ll->n_cation : ll->n_anion;
        const int32_t* la = k == 0 ? ll->cation : ll->anion;
        const int nb = k == 0 ? rl->n_anion : rl->n_cation;
        const int32_t* rb = k == 0 ? rl->anion : rl->cation;
        for (int a = 0; a < na; ++a)
            for (int b = 0; b < nb; ++b) {
                double dv[3];
                v_sub(x + 3 * la[a], rec_xyz + 3 * rb[b], dv);
                const double d = v_norm(dv);
                fl[2 + k] -= ramp_down(d, sf->ionic[k][0], sf->ionic[k][1]);
                if (d > 0.0) gacc(G, la[a], dv, -sk * ramp_down_d(d, sf->ionic[k][0], sf->ionic[k][1]) / d);
            }
    }
    /* cation-pi (scorer.cpp:370-462) */
    for (int k = 0; k < 2; ++k) {
        const double sk = g * w[PXD_W_COEF + PXD_TERM_PI_CATION] * w[PXD_W_PICAT + k];
        const int nr = k == 0 ? rl->n_ring5 : rl->n_ring6;
        const int32_t* rr = k == 0 ? rl->ring5 : rl->ring6;
        for (int r = 0; r < nr; ++r) {
            double c[3];
            ring_centroid(rec_xyz, rr + 6 * r, c);
            for (int a = 0; a < ll->n_cation; ++a) {
                const int i = ll->cation[a];
                double dv[3];
                v_sub(x + 3 * i, c, dv);
                const double d = v_norm(dv);
                fl[4 + k] -= ramp_down(d, sf->picat[k][0], sf->picat[k][1]);
                if (d > 0.0) gacc(G, i, dv, -sk * ramp_down_d(d, sf->picat[k][0], sf->picat[k][1]) / d);
            }
        }
    }
    for (int k = 2; k < 4; ++k) {
        const double sk = g * w[PXD_W_COEF + PXD_TERM_PI_CATION] * w[PXD_W_PICAT + k];
        const int nr = k == 2 ? ll->n_ring5 : ll->n_ring6;
        const int32_t* lr = k == 2 ? ll->ring5 : ll->ring6;
        for (int r = 0; r < nr; ++r) {
            double c[3], gc[3] = {0, 0, 0}, zero[3] = {0, 0, 0};
            ring_centroid(x, lr + 6 * r, c);
            for (int b = 0; b < rl->n_cation; ++b) {
                double dv[3];
                v_sub(c, rec_xyz + 3 * rl->cation[b], dv);
                const double d = v_norm(dv);
                fl[4 + k] -= ramp_down(d, sf->picat[k][0], sf->picat[k][1]);
                if (d > 0.0) {
                    const double q = -sk * ramp_down_d(d, sf->picat[k][0], sf->picat[k][1]) / d;
                    for (int u = 0; u < 3; ++u) gc[u] += q * dv[u];
                }
            }
            ring_backward(x, lr + 6 * r, gc, zero, G);
        }
    }
    /* pi stacking (scorer.cpp:638-724) */
    for (int q = 0; q < 2; ++q) {
        const double center = q == 0 ? 0.0 : 90.0;
        for (int lk = 0; lk < 2; ++lk) {      /* ligand ring5, ring6 */
            const int nlr = lk == 0 ? ll->n_ring5 : ll->n_ring6;
            const int32_t* lr = lk == 0 ? ll->ring5 : ll->ring6;
            for (int j = 0; j < nlr; ++j) {
                double lc[3], ln[3], glc[3] = {0, 0, 0}, gln[3] = {0, 0, 0};
                ring_centroid(x, lr + 6 * j, lc);
                ring_normal(x, lr + 6 * j, ln);
                for (int rk = 0; rk < 2; ++rk) {  /* receptor ring5, ring6 */
                    const int k = 2 * lk + rk;     /* l5r5 l5r6 l6r5 l6r6 */
                    const double sk = g * w[PXD_W_COEF + PXD_TERM_F2F + q] * w[PXD_W_STACK + 4 * q + k];
                    const int nrr = rk == 0 ? rl->n_ring5 : rl->n_ring6;
                    const int32_t* rr = rk == 0 ? rl->ring5 : rl->ring6;
                    for (int i = 0; i < nrr; ++i) {
                        double rc[3], rn[3];
                        ring_centroid(rec_xyz, rr + 6 * i, rc);
                        ring_normal(rec_xyz, rr + 6 * i, rn);
                        fl[8 + 4 * q + k] +=
                            stack_pair_diff(rc, rn, lc, ln, sf->stack[q][k], center, sk, G ? glc : NULL, gln);
                    }
                }
                ring_backward(x, lr + 6 * j, glc, gln, G);
            }
        }
    }
    /* hydrogen bonds (scorer.cpp:464-577) */
    {
        const double shb = g * w[PXD_W_COEF + PXD_TERM_HBOND] * w[PXD_W_HBOND_SCALE];
        for (int c = 0; c < 2; ++c) {  /* ligand donors x receptor acceptors */
            const int nd = c == 0 ? ll->n_don_charged : ll->n_don_neutral;
            const int32_t* dl = c == 0 ? ll->don_charged : ll->don_neutral;
            for (int a = 0; a < nd; ++a) {
                double gd[3] = {0, 0, 0}, gh[3] = {0, 0, 0}, gx[3] = {0, 0, 0};
                for (int u = 0; u < 2; ++u) {
                    const int na = u == 0 ? rl->n_acc_charged : rl->n_acc_neutral;
                    const int32_t* al = u == 0 ? rl->acc_charged : rl->acc_neutral;
                    const int k = 2 * c + u;
                    for (int b = 0; b < na; ++b)
                        fl[16 + k] += hbond_pair_diff(x + 3 * dl[2 * a], x + 3 * dl[2 * a + 1], rec_xyz + 3 * al[b],
                                                      sf->hbond[k], shb * w[PXD_W_HBOND + k], gd, gh, gx);
                }
                gacc(G, dl[2 * a], gd, 1.0);
                gacc(G, dl[2 * a + 1], gh, 1.0);
            }
        }
        for (int u = 0; u < 2; ++u) {  /* ligand acceptors x receptor donors */
            const int na = u == 0 ? ll->n_acc_charged : ll->n_acc_neutral;
            const int32_t* al = u == 0 ? ll->acc_charged : ll->acc_neutral;
            for (int a = 0; a < na; ++a) {
                double ga[3] = {0, 0, 0}, gd[3] = {0, 0, 0}, gh[3] = {0, 0, 0};
                for (int c = 0; c < 2; ++c) {
                    const int nd = c == 0 ? rl->n_don_charged : rl->n_don_neutral;
                    const int32_t* dl = c == 0 ? rl->don_charged : rl->don_neutral;
                    const int k = 4 + 2 * c + u;
                    for (int b = 0; b < nd; ++b)
                        fl[16 + k] += hbond_pair_diff(rec_xyz + 3 * dl[2 * b], rec_xyz + 3 * dl[2 * b + 1], x + 3 * al[a],
                                                      sf->hbond[k], shb * w[PXD_W_HBOND + k], gd, gh, ga);
                }
                gacc(G, al[a], ga, 1.0);
            }
        }
    }
    /* torsion strain (scorer.cpp:579-613) */
    {
        static const double per[4] = {1.0, 2.0, 3.0, 4.0};
        static const double ph[4] = {0.0, 3.141592653589793, 0.0, 3.141592653589793};
        const double sts = g * w[PXD_W_COEF + PXD_TERM_TSTRAIN];
        for (int e = 0; e < ll->n_tstrain; ++e) {
            const double* co = ll->tstrain_coefs + 4 * e;
            int cnt = 0;
            for (int q = ll->tstrain_offsets[e]; q < ll->tstrain_offsets[e + 1]; ++q) {
                if (ll->tstrain_quads[4 * q] == ll->tstrain_quads[4 * q + 1]) break;
                ++cnt;
            }
            if (cnt == 0) continue;
            double tmp = 0.0;
            for (int j = 0; j < cnt; ++j) {
                const int32_t* a = ll->tstrain_quads + 4 * (ll->tstrain_offsets[e] + j);
                double gi[3], gj[3], gk[3], gl[3];
                const double th = po_dihedral_and_gradient(x + 3 * a[0], x + 3 * a[1], x + 3 * a[2], x + 3 * a[3],
                                                           gi, gj, gk, gl);
                double df = 0.0;
                for (int m = 0; m < 4; ++m) {
                    tmp += (1 + cos(th * per[m] - ph[m])) * co[m];
                    df -= per[m] * sin(th * per[m] - ph[m]) * co[m];
                }
                const double k = sts * df / cnt;
                gacc(G, a[0], gi, k);
                gacc(G, a[1], gj, k);
                gacc(G, a[2], gk, k);
                gacc(G, a[3], gl, k);
            }
            fl[25] += tmp / cnt;
        }
    }
    fl[26] = -1.0 / (2.620643 + ll->n_rotatable);
    if (f) memcpy(f, fl, sizeof(fl));
    if (dw) po_combine_grad(w, fl, g, dw);
    return po_combine_features(w, fl);
}
