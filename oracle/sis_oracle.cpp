/*
 * sis_oracle.cpp -- CPU FP64 restatement of the SIS force/integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY (correctness oracle and timed CPU baseline).
 * Never linked into, loaded by or called from the product library.
 *
 * Every routine follows one Fortran routine of the reference (file:line given
 * at each function).  Arithmetic keeps the reference's expression order; the
 * library is compiled with -ffp-contract=off so that no multiply-add is fused
 * (the neighbour-list distance test then rounds exactly as an unfused FP64
 * evaluation of dot_product(v,v) does).  gfortran's norm2 is a scaled
 * algorithm; here sqrt(x*x+y*y+z*z) is used, which can differ from it in the
 * last bit.
 */
#include "sis_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* const_phys.F90:5-13 */
const double PI = 4.0 * atan(1.0);
const double EPS0 = 8.8541878128e-12;
const double ELE = 1.602176634e-19;
const double BOLTZ_J = 1.380649e-23;
const double N_AVO = 6.02214076e23;
const double KCAL2JOUL = 4184.0;
const double JOUL2KCAL = 1.0 / KCAL2JOUL;
const double JOUL2KCAL_MOL = JOUL2KCAL * N_AVO;
const double BOLTZ_KCAL_MOL = BOLTZ_J * JOUL2KCAL_MOL;

/* const_idx.F90: SEQT (A=0,U=1,G=2,C=3,D=4), BPT (GC=1,AU=2,GU=3,CG=4,UA=5,UG=6), MOLT */
enum { SA = 0, SU = 1, SG = 2, SC = 3, SD = 4 };
enum { GC = 1, AU = 2, GU = 3, CG = 4, UA = 5, UG = 6 };
enum { MOLT_RNA = 1, MOLT_CIRC = 2 };

/* const_idx.F90 is_complement */
bool is_complement(int s1, int s2) {
    if (s1 == SA) return s2 == SU;
    if (s1 == SU) return s2 == SA || s2 == SG;
    if (s1 == SG) return s2 == SC || s2 == SU;
    if (s1 == SC) return s2 == SG;
    return false;
}

/* const_idx.F90 NNT enumeration order (1..21) and char2nnt aliases */
int seqt2nnt(int i, int j, int k, int l) {
    static const char C[5] = {'A', 'U', 'G', 'C', 'D'};
    char s[6] = {C[i], C[j], '_', C[k], C[l], 0};
    static const char *names[21][2] = {
        {"GC_CG", ""},      {"CC_GG", "GG_CC"}, {"GA_CU", "UC_AG"}, {"CG_GC", ""},
        {"AC_UG", "GU_CA"}, {"CA_GU", "UG_AC"}, {"AG_UC", "CU_GA"}, {"UA_AU", ""},
        {"AU_UA", ""},      {"AA_UU", "UU_AA"}, {"GC_UG", "GU_CG"}, {"CU_GG", "GG_UC"},
        {"GG_CU", "UC_GG"}, {"CG_GU", "UG_GC"}, {"AU_UG", "GU_UA"}, {"GA_UU", "UU_AG"},
        {"UG_GU", ""},      {"UA_GU", "UG_AU"}, {"GG_UU", "UU_GG"}, {"GU_UG", ""},
        {"AG_UU", "UU_GA"}};
    for (int n = 0; n < 21; ++n)
        if (strcmp(s, names[n][0]) == 0 || (names[n][1][0] && strcmp(s, names[n][1]) == 0)) return n + 1;
    return 0; /* char2nnt leaves the result undefined; never reached for complementary stacks */
}

struct BPP { /* var_potential.F90:63-80 basepair_parameters */
    double cutoff_ddist, U0, bond_k, bond_r;
    double angl_k1, angl_k2, angl_k3, angl_k4;
    double angl_theta1, angl_theta2, angl_theta3, angl_theta4;
    double dihd_k1, dihd_k2, dihd_phi1, dihd_phi2;
};

struct Rep {
    std::vector<double> xyz, velos, accels, xyz_move;
    std::vector<int> wca_mp, ele_mp, bp_mp; /* 1-based bead indices */
    std::vector<double> bp_coef;
    std::vector<double> ene_bp;
    std::vector<uint8_t> bp_status, bp_status_MC;
    double tempK, ionstr;
    double ele_coef, lambdaD, ele_cutoff, diele, diele_dTcoef;
    std::vector<double> md_coef_rep;
};

} // namespace

struct or_mt {
    uint32_t st[624];
    int i;
    /* rnd_boxmuller.F90 saved spare */
    bool stored;
    double stored_value;
};

struct or_system {
    or_params p;
    int nmp, nchains, nrep;
    std::vector<int> nmp_chain, moltype, chain_start; /* chain_start: 0-based first bead */
    std::vector<int> seq;                           /* per bead */
    std::vector<int> lmp, ichain;                   /* 1-based local index, 0-based chain */
    std::vector<uint8_t> has_charge;
    bool pbc;
    double box[3], box_half[3];
    BPP bpp[7]; /* 1..6 */
    double bp_cutoff_dist;
    double bp3_dH[469], bp3_dS[469];
    int bp3_hash[4097];
    std::vector<int> bond_mp, angl_mp, dih_mp;
    std::vector<double> mass, fric, md_coef;
    std::vector<char> frozen; /* [Freeze]: is_frozen per bead (empty: none) */
    std::vector<Rep> rep;
    bool flg_bp_energy;
    int64_t nrebuild;
    int64_t istep = 0;            /* MD steps taken (job_md.F90 istep) */
    bool mc_now = false;          /* the next force evaluation runs the base-pair MC */
    std::vector<double> mc_draws; /* draws consumed by the last base-pair MC */
    std::vector<or_mt> mts;
    or_mt *spare_owner; /* the spare of rnd_boxmuller is shared by all replicas */
    bool spare_stored;
    double spare_value;
    /* optional terms, force.F90:62-75 / energy_sumup.F90:47-52 */
    bool stage = false;
    double stage_sigma = 0.0, stage_eps = 0.0;
    int rg_pott = 0;               /* 0 off, 1 harmonic, 2 flat-bottomed (const_idx.F90 POTT) */
    double rg_k = 0.0;
    std::vector<double> rg0;       /* per replica (bias_rg_0) */
    std::vector<int> rest_id;      /* [n][3]: imp, jmp (1-based), type 1 both beads, 2 subject only */
    std::vector<double> rest_para; /* [n][4]: eps, d, s, rcut (rest_sigb_para, rest_sigb_rcut) */
    std::vector<int> dcf_pairs;    /* [n][2] twz_DCF_pairs */
    std::vector<double> dcf_f;     /* [nrep][n][3] twz_DCF_forces */
    std::vector<int> fr_pairs;     /* [n][2] twz_FR_pairs */
    std::vector<double> fr_k;      /* [n][2] twz_FR_k */
    std::vector<double> fr_init, fr_velo; /* [n][2][3] twz_FR_init, twz_FR_velo */
    /* base pairs restricted to a given secondary structure (read_ss.F90 sets
     * bp_map from a ct/bpseq/bpl file; init_bp.F90:207-209 skips other pairs),
     * and the [Bias_SS] constant pull (force_bp_triplet.F90:85-92) */
    bool ss_on = false;
    std::vector<std::vector<int>> ss_part; /* per bead (0-based): 1-based partners */
    bool bias_ss = false;
    double bias_ss_force = 0.0;           /* kcal/mol/A */
};

namespace {

inline void pbc_vec_d(const or_system *s, const double *a, const double *b, double *v) {
    /* pbc.F90:140-165: single-shift minimum image */
    v[0] = a[0] - b[0];
    v[1] = a[1] - b[1];
    v[2] = a[2] - b[2];
    if (!s->pbc) return;
    for (int i = 0; i < 3; ++i) {
        if (v[i] > s->box_half[i])
            v[i] = v[i] - s->box[i];
        else if (v[i] < -s->box_half[i])
            v[i] = v[i] + s->box[i];
    }
}
inline double dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline double norm2(const double *a) { return sqrt(dot(a, a)); }
inline void cross(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
inline const double *X(const or_system *s, int irep, int imp1) { return &s->rep[irep].xyz[3 * (imp1 - 1)]; }

/* init_bp.F90:352-378 bp3_hash_key */
int bp3_hash_key(int w, int x, int u, int z, int y, int v) {
    int a, b, c, d, e, f;
    if (x < y) {
        a = w; b = x; c = u; d = z; e = y; f = v;
    } else {
        f = w; e = x; d = u; c = z; b = y; a = v;
    }
    return 1 + a + b * 4 + c * 16 + d * 64 + e * 256 + f * 1024;
}

/* init_bp.F90:39-172: NN triplet table (model 5) */
void init_bp3_tables(or_system *s) {
    const or_params &p = s->p;
    for (int k = 0; k <= 4096; ++k) s->bp3_hash[k] = 0;
    for (int k = 0; k <= 468; ++k) s->bp3_dH[k] = s->bp3_dS[k] = 0.0;
    if (p.bp_model != 5) return;
    int h = 0;
    for (int x = 0; x <= 2; ++x)
        for (int y = x + 1; y <= 3; ++y) {
            if (!is_complement(x, y)) continue;
            for (int w = 0; w <= 3; ++w)
                for (int z = 0; z <= 3; ++z) {
                    bool comp_wz = is_complement(w, z);
                    double dH, dS;
                    if (comp_wz) {
                        dH = 0.5 * (p.nn_dH[seqt2nnt(w, x, z, y) - 1] - p.dH0);
                        dS = 0.5 * (p.nn_dS[seqt2nnt(w, x, z, y) - 1] - p.dS0);
                    } else {
                        dH = 0.0;
                        dS = 0.0;
                    }
                    for (int u = 0; u <= 3; ++u)
                        for (int v = 0; v <= 3; ++v) {
                            bool comp_uv = is_complement(u, v);
                            if (!comp_wz && !comp_uv) continue;
                            h = h + 1;
                            int i = bp3_hash_key(w, x, u, z, y, v);
                            s->bp3_hash[i] = h;
                            if (comp_uv) {
                                s->bp3_dH[h] = dH + 0.5 * (p.nn_dH[seqt2nnt(x, u, y, v) - 1] - p.dH0);
                                s->bp3_dS[h] = (dS + 0.5 * (p.nn_dS[seqt2nnt(x, u, y, v) - 1] - p.dS0)) * 1.0e-3;
                            } else {
                                s->bp3_dH[h] = dH;
                                s->bp3_dS[h] = dS * 1.0e-3;
                            }
                            if (p.nnend) {
                                /* init_bp.F90:92-163 end effects.  NNENDT: 1 AUonAU 2 AUonCG 3 AUonGU
                                 * 4 GUonCG 5 GUonAU 6 GUonGU */
                                auto isAU = [](int a, int b) { return (a == SA && b == SU) || (a == SU && b == SA); };
                                auto isGC = [](int a, int b) { return (a == SG && b == SC) || (a == SC && b == SG); };
                                auto isGU = [](int a, int b) { return (a == SG && b == SU) || (a == SU && b == SG); };
                                int o1 = -1, o2 = -1; /* the paired neighbour (o1,o2) */
                                if (comp_wz && !comp_uv) {
                                    o1 = w; o2 = z;
                                } else if (!comp_wz && comp_uv) {
                                    o1 = u; o2 = v;
                                }
                                if (o1 >= 0) {
                                    int k = 0;
                                    if (isAU(x, y)) {
                                        if (isAU(o1, o2)) k = 1;
                                        else if (isGC(o1, o2)) k = 2;
                                        else if (isGU(o1, o2)) k = 3;
                                    } else if (isGU(x, y)) {
                                        if (isAU(o1, o2)) k = 5;
                                        else if (isGC(o1, o2)) k = 4;
                                        else if (isGU(o1, o2)) k = 6;
                                    }
                                    if (k > 0) {
                                        s->bp3_dH[h] = s->bp3_dH[h] + p.nnend_dH[k - 1] - p.dHend0;
                                        s->bp3_dS[h] = s->bp3_dS[h] + (p.nnend_dS[k - 1] - p.dSend0) * 1.0e-3;
                                    }
                                }
                            }
                        }
                }
        }
}

/* init_bp.F90:184-313 evaluated for one pair imp<jmp (1-based).  Returns the
 * pair type (bp_map) and writes bp3 (bp3_map).  No ct/bpseq/bpl input. */
int bp_candidate(const or_system *s, int imp, int jmp, int *bp3) {
    *bp3 = 0;
    const int model = s->p.bp_model, min_loop = s->p.bp_min_loop;
    int i = s->lmp[imp - 1], ic = s->ichain[imp - 1];
    int j = s->lmp[jmp - 1], jc = s->ichain[jmp - 1];
    int ni = s->nmp_chain[ic], nj = s->nmp_chain[jc];
    int i_pre = i - 1, i_nxt = i + 1, j_pre = j - 1, j_nxt = j + 1;
    bool i_circ, j_circ;
    if (s->moltype[ic] == MOLT_CIRC) {
        i_circ = true;
        if (i == 1) i_pre = ni;
        if (i == ni) i_nxt = 1;
    } else {
        i_circ = false;
        if (i == 1 || i == ni) return 0;
    }
    if (s->moltype[jc] == MOLT_CIRC) {
        j_circ = true;
        if (j == 1) j_pre = nj;
        if (j == nj) j_nxt = 1;
    } else {
        j_circ = false;
        if (j == 1 || j == nj) return 0;
    }
    auto sq = [&](int l, int c) { return s->seq[s->chain_start[c] + l - 1]; };
    bool pair_ipre_jnxt = is_complement(sq(i_pre, ic), sq(j_nxt, jc));
    bool pair_inxt_jpre = is_complement(sq(i_nxt, ic), sq(j_pre, jc));
    if (!i_circ && i_pre == 1) pair_ipre_jnxt = false;
    if (!j_circ && j_nxt == nj) pair_ipre_jnxt = false;
    if (!i_circ && i_nxt == ni) pair_inxt_jpre = false;
    if (!j_circ && j_pre == 1) pair_inxt_jpre = false;
    if (ic == jc) {
        if (i + min_loop >= j) return 0;
        if (i + 1 + min_loop >= j - 1) pair_inxt_jpre = false;
        if (i_circ) {
            if (j + min_loop >= i + ni) return 0;
            if (j + 1 + min_loop >= i - 1 + ni) pair_ipre_jnxt = false;
        }
    }
    if (model == 3 || model == 4 || model == 5)
        if (!pair_ipre_jnxt && !pair_inxt_jpre) return 0;
    int si = sq(i, ic), sj = sq(j, jc), type = 0;
    if (si == SG && sj == SC) type = GC;
    else if (si == SC && sj == SG) type = CG;
    else if (si == SA && sj == SU) type = AU;
    else if (si == SU && sj == SA) type = UA;
    else if (si == SG && sj == SU) type = GU;
    else if (si == SU && sj == SG) type = UG;
    if (model == 5) {
        int key;
        if (!pair_ipre_jnxt)
            key = bp3_hash_key(SU, si, sq(i_nxt, ic), SU, sj, sq(j_pre, jc));
        else if (!pair_inxt_jpre)
            key = bp3_hash_key(sq(i_pre, ic), si, SU, sq(j_nxt, jc), sj, SU);
        else
            key = bp3_hash_key(sq(i_pre, ic), si, sq(i_nxt, ic), sq(j_nxt, jc), sj, sq(j_pre, jc));
        *bp3 = s->bp3_hash[key];
    } else {
        *bp3 = type;
    }
    return type;
}

/* set_ele.F90:1-99 (default constants, not _HTN_CONSISTENT) */
void set_ele(or_system *s, int irep) {
    Rep &r = s->rep[irep];
    const double MM_A = 87.740, MM_B = -0.40008, MM_C = 9.398e-4, MM_D = -1.410e-6;
    double Tc;
    if (s->p.temp_independent == 0) {
        Tc = r.tempK - 273.15;
        r.diele = MM_A + MM_B * Tc + MM_C * Tc * Tc + MM_D * Tc * Tc * Tc;
        r.diele_dTcoef = 0.0;
    } else {
        Tc = s->p.tempK_ref - 273.15;
        r.diele = MM_A + MM_B * Tc + MM_C * Tc * Tc + MM_D * Tc * Tc * Tc;
        r.diele_dTcoef = 1.0 + s->p.tempK_ref / r.diele * (MM_B + 2.0 * MM_C * Tc + 3.0 * MM_D * Tc * Tc);
    }
    double lb = ELE * ELE / (4.0 * PI * EPS0 * r.diele * BOLTZ_J * r.tempK) * 1.0e10;
    double Zp = s->p.length_per_charge / lb;
    r.ele_coef = JOUL2KCAL_MOL * 1.0e10 * (ELE * ELE) / (4.0 * PI * EPS0 * r.diele);
    r.ele_coef = r.ele_coef * (Zp * Zp);
    r.lambdaD = 1.0e10 * sqrt((1.0e-3 * EPS0 * r.diele * BOLTZ_J) / (2.0 * N_AVO * (ELE * ELE))) * sqrt(r.tempK / r.ionstr);
    /* init_ele.F90:81-90 */
    if (s->p.ele_cutoff_type == 1)
        r.ele_cutoff = s->p.ele_cutoff_inp;
    else
        r.ele_cutoff = s->p.ele_cutoff_inp * r.lambdaD;
}

/* job_md.F90:94-133 friction and masses; set_md_coef job_md.F90:700-767 */
void set_md_coef(or_system *s) {
    const int n = s->nmp;
    s->mass.assign(n, 0.0);
    s->fric.assign(n, 0.0);
    s->md_coef.assign(3 * n, 0.0);
    const double radius = 10.0;
    double v;
    if (s->p.integrator == 1)
        v = s->p.viscosity_Pas * sqrt(1.0e3 / KCAL2JOUL) * N_AVO * 1.0e-20;
    else
        v = (JOUL2KCAL_MOL * 1.0e-18) * s->p.viscosity_Pas;
    for (int i = 0; i < n; ++i) {
        s->fric[i] = 6.0 * PI * v * radius;
        switch (s->seq[i]) {
        case SA: s->mass[i] = 328.212; break;
        case SG: s->mass[i] = 344.212; break;
        case SC: s->mass[i] = 304.182; break;
        case SU: s->mass[i] = 305.164; break;
        default: s->mass[i] = 320.443; break;
        }
    }
    const double dt = s->p.dt;
    for (int i = 0; i < n; ++i) {
        if (s->p.integrator == 1) {
            double c1 = 0.5 * dt * s->fric[i] / s->mass[i];
            double c2 = sqrt(1.0 / (1.0 + c1));
            s->md_coef[3 * i + 0] = (1.0 - c1) / (1.0 + c1);
            s->md_coef[3 * i + 1] = c2 * dt / s->mass[i];
            s->md_coef[3 * i + 2] = c2 * dt;
        } else {
            s->md_coef[3 * i + 0] = dt / s->fric[i];
        }
    }
    for (int r = 0; r < s->nrep; ++r) {
        Rep &R = s->rep[r];
        R.md_coef_rep.assign(n, 0.0);
        for (int i = 0; i < n; ++i) {
            if (s->p.integrator == 1) {
                double c1 = 0.5 * dt * s->fric[i] / s->mass[i];
                double c2 = sqrt(1.0 / (1.0 + c1));
                R.md_coef_rep[i] = 0.5 * c2 / s->mass[i] * sqrt(2.0 * s->fric[i] * BOLTZ_KCAL_MOL * R.tempK * dt);
            } else {
                R.md_coef_rep[i] = sqrt(2.0 * BOLTZ_KCAL_MOL * R.tempK * dt / s->fric[i]);
            }
        }
    }
    /* job_md.F90:713-729,745-748: a frozen bead's position coefficient is
     * zero (GJF-2GJ sqrt(b) h; Ermak-McCammon h/gamma and its noise) */
    if (!s->frozen.empty()) {
        for (int i = 0; i < n; ++i) {
            if (!s->frozen[i]) continue;
            if (s->p.integrator == 1) {
                s->md_coef[3 * i + 2] = 0.0;
            } else {
                s->md_coef[3 * i + 0] = 0.0;
                for (int r = 0; r < s->nrep; ++r) s->rep[r].md_coef_rep[i] = 0.0;
            }
        }
    }
}

/* pbc.F90:196-226 pbc_wrap: into [0, L) */
void pbc_wrap(or_system *s, int irep) {
    Rep &r = s->rep[irep];
    for (int imp = 0; imp < s->nmp; ++imp)
        for (int i = 0; i < 3; ++i) {
            double x = r.xyz[3 * imp + i];
            double bmax = s->box[i], bmin = 0.0;
            if (x > bmax)
                r.xyz[3 * imp + i] = x - s->box[i] * (double)((long long)((x - bmax) / s->box[i]) + 1);
            else if (x < bmin)
                r.xyz[3 * imp + i] = x + s->box[i] * (double)((long long)((bmin - x) / s->box[i]) + 1);
        }
}

} // namespace

/* ------------------------------------------------------------------ setup */
extern "C" or_system *or_create(int32_t nchains, const int32_t *chain_len, const int32_t *moltype,
                                const int32_t *seq, const uint8_t *has_charge, int32_t nrep,
                                const double *tempK, const double *ionic_strength, const double *pbc_box,
                                const or_params *p) {
    or_system *s = new or_system();
    s->p = *p;
    s->nchains = nchains;
    s->nrep = nrep;
    s->nmp = 0;
    for (int c = 0; c < nchains; ++c) {
        s->nmp_chain.push_back(chain_len[c]);
        s->moltype.push_back(moltype[c]);
        s->chain_start.push_back(s->nmp);
        for (int l = 1; l <= chain_len[c]; ++l) {
            s->lmp.push_back(l);
            s->ichain.push_back(c);
        }
        s->nmp += chain_len[c];
    }
    s->seq.assign(seq, seq + s->nmp);
    s->has_charge.assign(has_charge, has_charge + s->nmp);
    s->pbc = pbc_box != nullptr;
    for (int i = 0; i < 3; ++i) {
        s->box[i] = s->pbc ? pbc_box[i] : 0.0;
        s->box_half[i] = 0.5 * s->box[i];
    }
    /* read_force_field.F90:160-260: GC/AU/GU as read, CG/UA/UG with k1<->k2, k3<->k4
     * swapped and the angles NOT swapped */
    for (int t = 0; t < 3; ++t) {
        const double *f = p->bp_ff[t];
        BPP b;
        b.cutoff_ddist = 0.0;
        b.U0 = f[0]; b.bond_k = f[1]; b.bond_r = f[2];
        b.angl_k1 = f[3]; b.angl_k2 = f[4]; b.angl_k3 = f[5]; b.angl_k4 = f[6];
        b.angl_theta1 = f[7]; b.angl_theta2 = f[8]; b.angl_theta3 = f[9]; b.angl_theta4 = f[10];
        b.dihd_k1 = f[11]; b.dihd_k2 = f[12]; b.dihd_phi1 = f[13]; b.dihd_phi2 = f[14];
        s->bpp[1 + t] = b;
        BPP r = b;
        r.angl_k1 = b.angl_k2; r.angl_k2 = b.angl_k1;
        r.angl_k3 = b.angl_k4; r.angl_k4 = b.angl_k3;
        s->bpp[4 + t] = r;
    }
    /* init_bp.F90:315-346 cutoffs */
    if (fabs(p->bp_cutoff_energy) <= 2.220446049250313e-16) {
        s->bp_cutoff_dist = 18.0;
        for (int t = 1; t <= 6; ++t) s->bpp[t].cutoff_ddist = s->bp_cutoff_dist - 13.8;
    } else {
        s->bp_cutoff_dist = 0.0;
        for (int t = 1; t <= 6; ++t) {
            s->bpp[t].cutoff_ddist = sqrt(log(fabs(10.0 / p->bp_cutoff_energy)) / s->bpp[t].bond_k);
            double cutoff = s->bpp[t].bond_r + s->bpp[t].cutoff_ddist;
            if (cutoff > s->bp_cutoff_dist) s->bp_cutoff_dist = cutoff;
        }
    }
    init_bp3_tables(s);
    /* list_local.F90:1-126 */
    for (int c = 0; c < nchains; ++c) {
        int n = chain_len[c], base = s->chain_start[c] + 1;
        for (int i = 1; i <= n - 1; ++i) {
            int imp = base + i - 1;
            s->bond_mp.push_back(imp);
            s->bond_mp.push_back(imp + 1);
            if (i != n - 1) {
                s->angl_mp.push_back(imp);
                s->angl_mp.push_back(imp + 1);
                s->angl_mp.push_back(imp + 2);
            }
            if (p->dih_type != 0 && i < n - 2) {
                for (int k = 0; k < 4; ++k) s->dih_mp.push_back(imp + k);
            }
        }
        if (moltype[c] == MOLT_CIRC) {
            int ini = base, end = base + n - 1;
            s->bond_mp.push_back(end); s->bond_mp.push_back(ini);
            int a1[3] = {end - 1, end, ini}, a2[3] = {end, ini, ini + 1};
            s->angl_mp.insert(s->angl_mp.end(), a1, a1 + 3);
            s->angl_mp.insert(s->angl_mp.end(), a2, a2 + 3);
            if (p->dih_type != 0) {
                int d1[4] = {end - 2, end - 1, end, ini}, d2[4] = {end - 1, end, ini, ini + 1},
                    d3[4] = {end, ini, ini + 1, ini + 2};
                s->dih_mp.insert(s->dih_mp.end(), d1, d1 + 4);
                s->dih_mp.insert(s->dih_mp.end(), d2, d2 + 4);
                s->dih_mp.insert(s->dih_mp.end(), d3, d3 + 4);
            }
        }
    }
    s->rep.resize(nrep);
    for (int r = 0; r < nrep; ++r) {
        Rep &R = s->rep[r];
        R.xyz.assign(3 * s->nmp, 0.0);
        R.velos.assign(3 * s->nmp, 0.0);
        R.accels.assign(3 * s->nmp, 0.0);
        R.xyz_move.assign(3 * s->nmp, 0.0);
        R.tempK = tempK[r];
        R.ionstr = ionic_strength[r];
        set_ele(s, r);
    }
    set_md_coef(s);
    s->flg_bp_energy = false;
    s->nrebuild = 0;
    s->mts.resize(nrep);
    for (int r = 0; r < nrep; ++r) {
        or_mt *m = or_mt_create(1 + r);
        s->mts[r] = *m;
        or_mt_destroy(m);
    }
    s->spare_stored = false;
    s->spare_value = 0.0;
    return s;
}

extern "C" void or_destroy(or_system *s) { delete s; }
extern "C" int32_t or_nmp(const or_system *s) { return s->nmp; }
extern "C" void or_set_xyz(or_system *s, int32_t r, const double *x) { memcpy(s->rep[r].xyz.data(), x, 24 * (size_t)s->nmp); }
extern "C" void or_get_xyz(const or_system *s, int32_t r, double *x) { memcpy(x, s->rep[r].xyz.data(), 24 * (size_t)s->nmp); }
extern "C" void or_set_velos(or_system *s, int32_t r, const double *x) { memcpy(s->rep[r].velos.data(), x, 24 * (size_t)s->nmp); }
extern "C" void or_get_velos(const or_system *s, int32_t r, double *x) { memcpy(x, s->rep[r].velos.data(), 24 * (size_t)s->nmp); }
extern "C" void or_set_accels(or_system *s, int32_t r, const double *x) { memcpy(s->rep[r].accels.data(), x, 24 * (size_t)s->nmp); }
extern "C" void or_get_accels(const or_system *s, int32_t r, double *x) { memcpy(x, s->rep[r].accels.data(), 24 * (size_t)s->nmp); }

extern "C" void or_set_temperature(or_system *s, int32_t irep, double tempK, double ionstr) {
    s->rep[irep].tempK = tempK;
    s->rep[irep].ionstr = ionstr;
    set_ele(s, irep);
    set_md_coef(s);
}

/* [Freeze] id_ranges, as 1-based bead numbers (the same in every replica) */
/* read_ss.F90: the pairs (imp, jmp), 1-based, that bp_map allows; n = 0
 * lifts the restriction */
extern "C" void or_set_ss_pairs(or_system *s, int32_t n, const int32_t *pairs) {
    s->ss_on = n > 0;
    s->ss_part.assign(s->nmp, {});
    for (int q = 0; q < n; ++q) {
        const int i = pairs[2 * q], j = pairs[2 * q + 1];
        if (i < 1 || j < 1 || i > s->nmp || j > s->nmp) continue;
        s->ss_part[i - 1].push_back(j);
        s->ss_part[j - 1].push_back(i);
    }
}
/* read_input.F90:1198-1217 [Bias_SS]: on, force in kcal/mol/A */
extern "C" void or_set_bias_ss(or_system *s, int32_t on, double force) {
    s->bias_ss = on != 0;
    s->bias_ss_force = force;
}

extern "C" void or_set_frozen(or_system *s, int32_t n, const int32_t *beads) {
    s->frozen.assign(s->nmp, 0);
    for (int q = 0; q < n; ++q)
        if (beads[q] >= 1 && beads[q] <= s->nmp) s->frozen[beads[q] - 1] = 1;
    set_md_coef(s);
}

extern "C" void or_get_ele(const or_system *s, int32_t irep, double *o) {
    const Rep &r = s->rep[irep];
    o[0] = r.ele_coef; o[1] = r.lambdaD; o[2] = r.ele_cutoff; o[3] = r.diele;
}
extern "C" void or_get_md_coef(const or_system *s, int32_t irep, double *o) {
    for (int i = 0; i < s->nmp; ++i) {
        o[4 * i + 0] = s->md_coef[3 * i + 0];
        o[4 * i + 1] = s->md_coef[3 * i + 1];
        o[4 * i + 2] = s->md_coef[3 * i + 2];
        o[4 * i + 3] = s->rep[irep].md_coef_rep[i];
    }
}
extern "C" void or_get_bp_paras(const or_system *s, double *o, double *cut) {
    for (int t = 1; t <= 6; ++t) memcpy(o + 16 * (t - 1), &s->bpp[t], sizeof(BPP));
    *cut = s->bp_cutoff_dist;
}
extern "C" void or_get_bp3_tables(const or_system *s, double *dH, double *dS) {
    for (int h = 1; h <= 468; ++h) {
        dH[h - 1] = s->bp3_dH[h];
        dS[h - 1] = s->bp3_dS[h];
    }
}
extern "C" double or_const(int32_t w) {
    switch (w) {
    case 0: return PI;
    case 1: return BOLTZ_KCAL_MOL;
    case 2: return JOUL2KCAL_MOL;
    default: return 0.0;
    }
}

/* ---------------------------------------------------------- neighbour list */
/* neighbor_list.F90:1-233.  The O(N^2) scan runs over rows (chain ic, chain
 * jc >= ic, a block of 64 beads i of ic) in parallel; each row appends to its
 * own buffers, which are joined in row order, so the lists come out in the
 * reference's serial (ic, jc, i, j) order whatever the thread count. */
namespace {
struct NlRow {
    int ic, jc, i0, i1;
};
struct NlOut {
    std::vector<int> wca, ele, bp;
    std::vector<double> coef;
};
} // namespace

extern "C" void or_neighbor_list(or_system *s, int32_t irep) {
    Rep &R = s->rep[irep];
    const or_params &p = s->p;
    if (s->pbc) pbc_wrap(s, irep);
    R.wca_mp.clear();
    R.ele_mp.clear();
    R.bp_mp.clear();
    R.bp_coef.clear();
    double ele_nl_cut2 = 0.0;
    if (p.flg_ele) {
        if (p.ele_cutoff_type == 2) R.ele_cutoff = p.ele_cutoff_inp * R.lambdaD;
        ele_nl_cut2 = (R.ele_cutoff + p.nl_margin) * (R.ele_cutoff + p.nl_margin);
    }
    const double wca_nl_cut2 = (p.wca_sigma + p.nl_margin) * (p.wca_sigma + p.nl_margin);
    /* neighbor_list.F90:89-93: with [Bias_SS] every allowed pair is listed
     * (the REAL(4) literal 9999999999.9 is 1e10 exactly) */
    const double bp_nl_cut2 =
        s->bias_ss ? (double)9999999999.9f : (s->bp_cutoff_dist + p.nl_margin) * (s->bp_cutoff_dist + p.nl_margin);
    std::vector<NlRow> rows;
    for (int ic = 0; ic < s->nchains; ++ic)
        for (int jc = ic; jc < s->nchains; ++jc)
            for (int i0 = 1; i0 <= s->nmp_chain[ic]; i0 += 64) rows.push_back({ic, jc, i0, std::min(i0 + 63, s->nmp_chain[ic])});
    std::vector<NlOut> out(rows.size());
#pragma omp parallel for schedule(dynamic, 16)
    for (long r = 0; r < (long)rows.size(); ++r) {
        const int ic = rows[r].ic, jc = rows[r].jc;
        NlOut &o = out[r];
        const int ni = s->nmp_chain[ic], nj = s->nmp_chain[jc];
        for (int i = rows[r].i0; i <= rows[r].i1; ++i) {
            const int imp = s->chain_start[ic] + i;
            const int iseq = s->seq[imp - 1];
            const int j_start = (ic == jc) ? i + 1 : 1;
            for (int j = j_start; j <= nj; ++j) {
                const int jmp = s->chain_start[jc] + j;
                const int jseq = s->seq[jmp - 1];
                double v[3];
                pbc_vec_d(s, X(s, irep, imp), X(s, irep, jmp), v);
                const double d2 = dot(v, v);
                if (iseq != SD && jseq != SD && d2 <= wca_nl_cut2) {
                    bool add = true;
                    if (ic == jc) {
                        if (i + 2 >= j) add = false;
                        else if (s->moltype[ic] == MOLT_CIRC && j + 2 >= i + ni) add = false;
                    }
                    if (add) {
                        o.wca.push_back(imp);
                        o.wca.push_back(jmp);
                    }
                }
                if (p.flg_ele && d2 <= ele_nl_cut2 && s->has_charge[imp - 1] && s->has_charge[jmp - 1]) {
                    bool add = true;
                    if (ic == jc) {
                        if (j == i + 1 && p.ele_excl_bond) add = false;
                        if (j == i + 2 && p.ele_excl_angle) add = false;
                        if (s->moltype[ic] == MOLT_CIRC) {
                            if (i == 1) {
                                if (j == ni && p.ele_excl_bond) add = false;
                                if (j == ni - 1 && p.ele_excl_angle) add = false;
                            } else if (i == 2) {
                                if (j == ni && p.ele_excl_angle) add = false;
                            }
                        }
                    }
                    if (add) {
                        o.ele.push_back(imp);
                        o.ele.push_back(jmp);
                    }
                }
                bool ss_ok = !s->ss_on;
                if (!ss_ok)
                    for (int jj : s->ss_part[imp - 1]) ss_ok |= jj == jmp;
                if (d2 <= bp_nl_cut2 && ss_ok) {
                    int bp3;
                    int type = bp_candidate(s, imp, jmp, &bp3);
                    if (bp3 > 0) {
                        int rec[7];
                        rec[0] = imp;
                        rec[1] = jmp;
                        rec[2] = (i == 1) ? imp + ni - 1 : imp - 1;
                        rec[3] = (j == 1) ? jmp + nj - 1 : jmp - 1;
                        rec[4] = (i == ni) ? imp + 1 - ni : imp + 1;
                        const int jend = p.bp_jnext_compat ? ni : nj; /* neighbor_list.F90:212 */
                        rec[5] = (j == jend) ? jmp + 1 - nj : jmp + 1;
                        rec[6] = type;
                        o.bp.insert(o.bp.end(), rec, rec + 7);
                        o.coef.push_back(s->bp3_dH[bp3]);
                        o.coef.push_back(s->bp3_dS[bp3]);
                    }
                }
            }
        }
    }
    for (const NlOut &o : out) {
        R.wca_mp.insert(R.wca_mp.end(), o.wca.begin(), o.wca.end());
        R.ele_mp.insert(R.ele_mp.end(), o.ele.begin(), o.ele.end());
        R.bp_mp.insert(R.bp_mp.end(), o.bp.begin(), o.bp.end());
        R.bp_coef.insert(R.bp_coef.end(), o.coef.begin(), o.coef.end());
    }
    const size_t nbp = R.bp_mp.size() / 7;
    R.ene_bp.assign(nbp, 0.0);
    R.bp_status.assign(nbp, 0);
    R.bp_status_MC.assign(nbp, 1);
    s->nrebuild++;
}

extern "C" int32_t or_get_list(const or_system *s, int32_t irep, int32_t kind, int32_t *out, int32_t cap) {
    const Rep &R = s->rep[irep];
    const std::vector<int> &L = kind == 0 ? R.wca_mp : kind == 1 ? R.ele_mp : R.bp_mp;
    const int w = kind == 2 ? 7 : 2;
    const int n = (int)(L.size() / w);
    const int m = std::min(n, cap);
    if (out && m > 0) memcpy(out, L.data(), sizeof(int) * (size_t)m * w);
    return n;
}
extern "C" int32_t or_get_bp_coef(const or_system *s, int32_t irep, double *out, int32_t cap) {
    const Rep &R = s->rep[irep];
    const int n = (int)(R.bp_coef.size() / 2);
    const int m = std::min(n, cap);
    if (out && m > 0) memcpy(out, R.bp_coef.data(), sizeof(double) * 2 * (size_t)m);
    return n;
}

/* ------------------------------------------------------------------ forces */
namespace {

inline void addf(double *F, int imp, const double *f, double sgn) {
    F[3 * (imp - 1) + 0] += sgn * f[0];
    F[3 * (imp - 1) + 1] += sgn * f[1];
    F[3 * (imp - 1) + 2] += sgn * f[2];
}

/* force_bond.F90:33-57 */
void force_bond(const or_system *s, int irep, double *F, int lo, int hi) {
    for (int ib = lo; ib < hi; ++ib) {
        int i1 = s->bond_mp[2 * ib], i2 = s->bond_mp[2 * ib + 1];
        double v[3], f[3];
        pbc_vec_d(s, X(s, irep, i1), X(s, irep, i2), v);
        double d = norm2(v);
        double delta = d - s->p.bond_r0;
        for (int k = 0; k < 3; ++k) f[k] = s->p.bond_k * delta / d * v[k];
        addf(F, i1, f, -1.0);
        addf(F, i2, f, +1.0);
    }
}

/* force_angl.F90:35-83 */
void force_angl(const or_system *s, int irep, double *F, int lo, int hi) {
    for (int ia = lo; ia < hi; ++ia) {
        int i1 = s->angl_mp[3 * ia], i2 = s->angl_mp[3 * ia + 1], i3 = s->angl_mp[3 * ia + 2];
        double v21[3], v32[3], f21[3], f32[3];
        pbc_vec_d(s, X(s, irep, i2), X(s, irep, i1), v21);
        pbc_vec_d(s, X(s, irep, i3), X(s, irep, i2), v32);
        double d21 = dot(v21, v21), d32 = dot(v32, v32), d2132 = dot(v32, v21);
        double cosine = -d2132 / sqrt(d21 * d32);
        if (fabs(cosine) > 1.0) cosine = copysign(1.0, cosine);
        double delta = acos(cosine) - s->p.angl_t0;
        double t = d21 * d32 - d2132 * d2132;
        if (t <= 1.0) t = 1.0;
        double f = s->p.angl_k * delta / sqrt(t);
        for (int k = 0; k < 3; ++k) {
            f21[k] = f * (v21[k] * (d2132 / d21) - v32[k]);
            f32[k] = f * (v32[k] * (d2132 / d32) - v21[k]);
        }
        addf(F, i1, f21, -1.0);
        double m[3] = {f21[0] - f32[0], f21[1] - f32[1], f21[2] - f32[2]};
        addf(F, i2, m, 1.0);
        addf(F, i3, f32, 1.0);
    }
}

/* force_angl_ReB.F90:36-74 */
void force_angl_reb(const or_system *s, int irep, double *F, int lo, int hi) {
    const double co0 = cos(s->p.angl_t0);
    for (int ia = lo; ia < hi; ++ia) {
        int i1 = s->angl_mp[3 * ia], i2 = s->angl_mp[3 * ia + 1], i3 = s->angl_mp[3 * ia + 2];
        double v12[3], v32[3], f1[3], f3[3];
        pbc_vec_d(s, X(s, irep, i1), X(s, irep, i2), v12);
        pbc_vec_d(s, X(s, irep, i3), X(s, irep, i2), v32);
        double d12 = dot(v12, v12), d32 = dot(v32, v32);
        double a1232 = sqrt(d12 * d32);
        double cosine = dot(v12, v32) / a1232;
        double omc = 1.0 - cosine * cosine;
        double f = -s->p.angl_k * (cosine - co0) * (1.0 - cosine * co0) / (omc * omc);
        for (int k = 0; k < 3; ++k) {
            f1[k] = f * (v32[k] / a1232 - cosine * v12[k] / d12);
            f3[k] = f * (v12[k] / a1232 - cosine * v32[k] / d32);
        }
        addf(F, i1, f1, 1.0);
        double m[3] = {f1[0] + f3[0], f1[1] + f3[1], f1[2] + f3[2]};
        addf(F, i2, m, -1.0);
        addf(F, i3, f3, 1.0);
    }
}

/* force_dih_cos.F90:19-60 and force_dih_exp.F90:36-95 */
void force_dih(const or_system *s, int irep, double *F, int lo, int hi) {
    const double coef1 = s->p.dih_k * s->p.dih_w, coef2 = -0.5 * s->p.dih_w;
    for (int id = lo; id < hi; ++id) {
        int i1 = s->dih_mp[4 * id], i2 = s->dih_mp[4 * id + 1], i3 = s->dih_mp[4 * id + 2], i4 = s->dih_mp[4 * id + 3];
        double vij[3], vkj[3], vkl[3], m[3], n[3], fi[3], fj[3], fk[3], fl[3];
        pbc_vec_d(s, X(s, irep, i1), X(s, irep, i2), vij);
        pbc_vec_d(s, X(s, irep, i3), X(s, irep, i2), vkj);
        pbc_vec_d(s, X(s, irep, i3), X(s, irep, i4), vkl);
        cross(vij, vkj, m);
        cross(vkj, vkl, n);
        double akj2 = dot(vkj, vkj), akj = sqrt(akj2);
        double dih = atan2(akj * dot(vij, n), dot(m, n));
        double pre;
        if (s->p.dih_type == 1)
            pre = -s->p.dih_k * sin(dih + s->p.dih_p0) * akj;
        else
            pre = coef1 * (dih - s->p.dih_p0) * exp(coef2 * ((dih - s->p.dih_p0) * (dih - s->p.dih_p0))) * akj;
        double mm = dot(m, m), nn = dot(n, n);
        for (int k = 0; k < 3; ++k) {
            fi[k] = -pre / mm * m[k];
            fl[k] = pre / nn * n[k];
        }
        double a = dot(vij, vkj) / akj2, b = dot(vkl, vkj) / akj2;
        for (int k = 0; k < 3; ++k) {
            fj[k] = (-1.0 + a) * fi[k] + (-b) * fl[k];
            fk[k] = (-a) * fi[k] + (-1.0 + b) * fl[k];
        }
        addf(F, i1, fi, 1.0);
        addf(F, i2, fj, 1.0);
        addf(F, i3, fk, 1.0);
        addf(F, i4, fl, 1.0);
    }
}

/* force_wca.F90:34-67 */
void force_wca(const or_system *s, int irep, double *F, int lo, int hi) {
    const Rep &R = s->rep[irep];
    const double sig2 = s->p.wca_sigma * s->p.wca_sigma;
    const double coef = 12.0 * s->p.wca_eps / sig2;
    for (int k = lo; k < hi; ++k) {
        int i1 = R.wca_mp[2 * k], i2 = R.wca_mp[2 * k + 1];
        double v[3];
        pbc_vec_d(s, X(s, irep, i1), X(s, irep, i2), v);
        double d2 = dot(v, v);
        if (d2 >= sig2) continue;
        d2 = sig2 / d2;
        double d4 = d2 * d2 * d2 * d2;
        double d7 = d4 * d2 * d2 * d2;
        double f[3];
        for (int c = 0; c < 3; ++c) f[c] = coef * (d7 - d4) * v[c];
        addf(F, i1, f, 1.0);
        addf(F, i2, f, -1.0);
    }
}

/* force_ele_DH.F90:39-82 */
void force_ele(const or_system *s, int irep, double *F, int lo, int hi) {
    const Rep &R = s->rep[irep];
    const double cutoff2 = R.ele_cutoff * R.ele_cutoff;
    const double rcdist = 1.0 / R.lambdaD;
    for (int k = lo; k < hi; ++k) {
        int i1 = R.ele_mp[2 * k], i2 = R.ele_mp[2 * k + 1];
        double v21[3];
        pbc_vec_d(s, X(s, irep, i2), X(s, irep, i1), v21);
        double dist2 = dot(v21, v21);
        if (dist2 > cutoff2) continue;
        double dist1 = sqrt(dist2);
        double rdist1 = 1.0 / dist1;
        double dvdw_dr = R.ele_coef * rdist1 * rdist1 * (rdist1 + rcdist) * exp(-dist1 * rcdist);
        double f[3] = {dvdw_dr * v21[0], dvdw_dr * v21[1], dvdw_dr * v21[2]};
        addf(F, i1, f, -1.0);
        addf(F, i2, f, 1.0);
    }
}

/* force_bp.F90:44-204 (model 1/3) and force_bp_triplet.F90:62-240 (model 4/5):
 * one record.  Returns true when the pair is formed (ene <= cutoff). */
bool bp_one(const or_system *s, int irep, int ibp, double tK, double *F, double *ene_out, double (*fout)[3] = nullptr,
            double *Fpull = nullptr) {
    const Rep &R = s->rep[irep];
    const int *rec = &R.bp_mp[7 * ibp];
    const int i1 = rec[0], i2 = rec[1], i3 = rec[2], i4 = rec[3], i5 = rec[4], i6 = rec[5];
    const BPP &b = s->bpp[rec[6]];
    const bool triplet = s->p.bp_model == 4 || s->p.bp_model == 5;
    double dG = 0.0;
    if (triplet) {
        dG = R.bp_coef[2 * ibp] - tK * R.bp_coef[2 * ibp + 1];
        if (dG >= 0.0) return false;
    }
    double v12[3], v13[3], v15[3], v42[3], v62[3], fb[6][3], fi[3], fk[3], fl[3], m[3], n[3];
    pbc_vec_d(s, X(s, irep, i1), X(s, irep, i2), v12);
    double d1212 = dot(v12, v12);
    double a12 = sqrt(d1212);
    double d = a12 - b.bond_r;
    if (fabs(d) > b.cutoff_ddist) {
        /* force_bp_triplet.F90:85-92 / force_bp_limit_triplet.F90:104-111: a
         * constant pull of i toward j outside the distance window */
        double *Fp = F ? F : Fpull;
        if (s->bias_ss && triplet && Fp) {
            double f[3];
            for (int k = 0; k < 3; ++k) f[k] = s->bias_ss_force / a12 * v12[k];
            addf(Fp, i1, f, -1.0);
            addf(Fp, i2, f, 1.0);
        }
        return false;
    }
    double u = b.bond_k * (d * d);
    for (int k = 0; k < 3; ++k) {
        fi[k] = (2.0 * b.bond_k * d / a12) * v12[k];
        fb[0][k] = fi[k];
        fb[1][k] = -fi[k];
    }
    pbc_vec_d(s, X(s, irep, i1), X(s, irep, i3), v13);
    pbc_vec_d(s, X(s, irep, i1), X(s, irep, i5), v15);
    pbc_vec_d(s, X(s, irep, i4), X(s, irep, i2), v42);
    pbc_vec_d(s, X(s, irep, i6), X(s, irep, i2), v62);
    double d1313 = dot(v13, v13), d4242 = dot(v42, v42), d1213 = dot(v12, v13), d1242 = dot(v12, v42);
    double d1215 = dot(v12, v15), d1515 = dot(v15, v15), d1262 = dot(v12, v62), d6262 = dot(v62, v62);
    double o13 = d1213 / d1212, o42 = d1242 / d1212, o15 = d1215 / d1212, o62 = d1262 / d1212;
    double cosine, pre;
    /* 3-1=2 */
    cosine = d1213 / (sqrt(d1313) * a12);
    d = acos(cosine) - b.angl_theta2;
    pre = 2.0 * b.angl_k2 * d / sqrt(d1313 * d1212 - d1213 * d1213);
    u = u + b.angl_k2 * (d * d);
    for (int k = 0; k < 3; ++k) {
        fi[k] = pre * (v12[k] - (d1213 / d1313 * v13[k]));
        fk[k] = pre * (v13[k] - (o13 * v12[k]));
        fb[0][k] = fb[0][k] - fi[k] - fk[k];
        fb[1][k] = fb[1][k] + fk[k];
        fb[2][k] = fi[k];
    }
    /* 1=2-4 */
    cosine = d1242 / (a12 * sqrt(d4242));
    d = acos(cosine) - b.angl_theta1;
    u = u + b.angl_k1 * (d * d);
    pre = 2.0 * b.angl_k1 * d / sqrt(d1212 * d4242 - d1242 * d1242);
    for (int k = 0; k < 3; ++k) {
        fi[k] = -pre * (v42[k] - (o42 * v12[k]));
        fk[k] = -pre * (v12[k] - (d1242 / d4242 * v42[k]));
        fb[0][k] = fb[0][k] + fi[k];
        fb[1][k] = fb[1][k] - fi[k] - fk[k];
        fb[3][k] = fk[k];
    }
    /* 5-1=2 */
    cosine = d1215 / (sqrt(d1515) * a12);
    d = acos(cosine) - b.angl_theta4;
    u = u + b.angl_k4 * (d * d);
    pre = 2.0 * b.angl_k4 * d / sqrt(d1515 * d1212 - d1215 * d1215);
    for (int k = 0; k < 3; ++k) {
        fi[k] = pre * (v12[k] - (d1215 / d1515 * v15[k]));
        fk[k] = pre * (v15[k] - (o15 * v12[k]));
        fb[0][k] = fb[0][k] - fi[k] - fk[k];
        fb[1][k] = fb[1][k] + fk[k];
        fb[4][k] = fi[k];
    }
    /* 1=2-6 */
    cosine = d1262 / (a12 * sqrt(d6262));
    d = acos(cosine) - b.angl_theta3;
    u = u + b.angl_k3 * (d * d);
    pre = 2.0 * b.angl_k3 * d / sqrt(d1212 * d6262 - d1262 * d1262);
    for (int k = 0; k < 3; ++k) {
        fi[k] = -pre * (v62[k] - (o62 * v12[k]));
        fk[k] = -pre * (v12[k] - (d1262 / d6262 * v62[k]));
        fb[0][k] = fb[0][k] + fi[k];
        fb[1][k] = fb[1][k] - fi[k] - fk[k];
        fb[5][k] = fk[k];
    }
    /* dihedral 4-2=1=3 */
    cross(v42, v12, m);
    cross(v12, v13, n);
    double dih = atan2(dot(v42, n) * a12, dot(m, n));
    d = dih + b.dihd_phi1;
    u = u + b.dihd_k1 * (1.0 + cos(d));
    pre = -b.dihd_k1 * sin(d) * a12;
    double mm = dot(m, m), nn = dot(n, n);
    for (int k = 0; k < 3; ++k) {
        fi[k] = pre / mm * m[k];
        fl[k] = -pre / nn * n[k];
    }
    for (int k = 0; k < 3; ++k) {
        fb[3][k] = fb[3][k] + fi[k];
        fb[1][k] = fb[1][k] + (-1.0 + o42) * fi[k] - (o13)*fl[k];
        fb[0][k] = fb[0][k] + (-1.0 + o13) * fl[k] - (o42)*fi[k];
        fb[2][k] = fb[2][k] + fl[k];
    }
    /* dihedral 6-2=1=5 */
    cross(v62, v12, m);
    cross(v12, v15, n);
    dih = atan2(dot(v62, n) * a12, dot(m, n));
    d = dih + b.dihd_phi2;
    u = u + b.dihd_k2 * (1.0 + cos(d));
    pre = -b.dihd_k2 * sin(d) * a12;
    mm = dot(m, m);
    nn = dot(n, n);
    for (int k = 0; k < 3; ++k) {
        fi[k] = pre / mm * m[k];
        fl[k] = -pre / nn * n[k];
    }
    for (int k = 0; k < 3; ++k) {
        fb[5][k] = fb[5][k] + fi[k];
        fb[1][k] = fb[1][k] + (-1.0 + o62) * fi[k] - (o15)*fl[k];
        fb[0][k] = fb[0][k] + (-1.0 + o15) * fl[k] - (o62)*fi[k];
        fb[4][k] = fb[4][k] + fl[k];
    }
    double ene = triplet ? b.U0 * dG * exp(-u) : b.U0 * exp(-u);
    if (ene <= s->p.bp_cutoff_energy) {
        *ene_out = ene;
        const int ids[6] = {i1, i2, i3, i4, i5, i6};
        for (int q = 0; q < 6; ++q) {
            double f[3] = {ene * fb[q][0], ene * fb[q][1], ene * fb[q][2]};
            if (F) addf(F, ids[q], f, 1.0);
            if (fout)
                for (int k = 0; k < 3; ++k) fout[q][k] = f[k];
        }
        return true;
    }
    return false;
}

/* force_bp_limit_triplet.F90:66-372: every record evaluated (records off the
 * window or above the energy cut stay off), then, while any nucleotide
 * carries more than max_bp_per_nt pairs: pick one of those nucleotides
 * uniformly (genrand_double3), shuffle its pairs (one genrand_double3 swap
 * per position), walk them keeping the candidate with probability
 * exp((E_j - E_keep) / kT) (genrand_double1), and delete the survivor.  The
 * remaining pairs' forces are added to F; their status is the mask of the
 * steps until the next Monte Carlo pass (job_md.F90:399-401).  Models 1 and 3
 * use the same removal on their energies: the reference's force_bp_limit.F90
 * reads the pair type from bp_mp(3,.) (a bead index) and is not restated. */
void bp_mc(or_system *s, int irep, double tK, double *F) {
    Rep &R = s->rep[irep];
    const int nbp = (int)R.bp_mp.size() / 7;
    std::vector<double> fr((size_t)nbp * 18, 0.0);
    std::vector<int> excess(s->nmp, -s->p.max_bp_per_nt);
    R.bp_status.assign(nbp, 0);
    R.ene_bp.assign(nbp, 0.0);
    for (int ibp = 0; ibp < nbp; ++ibp) {
        double e;
        if (bp_one(s, irep, ibp, tK, nullptr, &e, (double(*)[3]) & fr[(size_t)18 * ibp], F)) {
            R.bp_status[ibp] = 1;
            R.ene_bp[ibp] = e;
            excess[R.bp_mp[7 * ibp] - 1]++;
            excess[R.bp_mp[7 * ibp + 1] - 1]++;
        }
    }
    const double beta = 1.0 / (BOLTZ_KCAL_MOL * tK);
    or_mt *mt = &s->mts[irep];
    s->mc_draws.clear();
    std::vector<int> list, seq;
    for (;;) {
        list.clear();
        for (int i = 0; i < s->nmp; ++i)
            if (excess[i] > 0) list.push_back(i + 1);
        if (list.empty()) break;
        double rnd = or_mt_double3(mt);
        s->mc_draws.push_back(rnd);
        const int nt = list[(int)ceil(rnd * (double)list.size()) - 1];
        seq.clear();
        for (int ibp = 0; ibp < nbp; ++ibp)
            if (R.bp_status[ibp] && (R.bp_mp[7 * ibp] == nt || R.bp_mp[7 * ibp + 1] == nt)) seq.push_back(ibp);
        const int m = (int)seq.size();
        for (int i = 0; i < m; ++i) {
            rnd = or_mt_double3(mt);
            s->mc_draws.push_back(rnd);
            std::swap(seq[i], seq[(int)ceil(rnd * (double)m) - 1]);
        }
        int del = seq[0];
        for (int i = 1; i < m; ++i) {
            const int j = seq[i];
            const double ratio = exp((R.ene_bp[j] - R.ene_bp[del]) * beta);
            rnd = or_mt_double1(mt);
            s->mc_draws.push_back(rnd);
            if (rnd < ratio) del = j;
        }
        R.bp_status[del] = 0;
        R.ene_bp[del] = 0.0;
        excess[R.bp_mp[7 * del] - 1]--;
        excess[R.bp_mp[7 * del + 1] - 1]--;
    }
    for (int ibp = 0; ibp < nbp; ++ibp) {
        if (!R.bp_status[ibp]) continue;
        for (int q = 0; q < 6; ++q) addf(F, R.bp_mp[7 * ibp + q], &fr[(size_t)18 * ibp + 3 * q], 1.0);
    }
    R.bp_status_MC = R.bp_status;
}

int nthreads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // namespace

/* The optional terms of force.F90:62-75 (term 7 here): force_stage.F90,
 * force_tweezers.F90 (istep: the step being taken, job_md.F90:362),
 * force_rg.F90 and force_restraint.F90. */
static void force_bias(or_system *s, int irep, double *forces, int64_t istep) {
    const Rep &R = s->rep[irep];
    const int n = s->nmp;
    if (s->stage) {
        const double coef = 24.0 * s->stage_eps / s->stage_sigma;
        const double small = DBL_EPSILON; /* const_phys.F90 SMALL_VALUE = epsilon(PI) */
        for (int i = 0; i < n; ++i) {
            double z = R.xyz[3 * i + 2];
            if (z < small) z = small;
            z = s->stage_sigma / z;
            const double z2 = z * z, z6 = z2 * z2 * z2, z7 = z6 * z, z13 = z6 * z7;
            forces[3 * i + 2] = forces[3 * i + 2] + coef * (2.0 * z13 - z7);
        }
    }
    const int ndcf = (int)s->dcf_pairs.size() / 2;
    for (int q = 0; q < ndcf; ++q) {
        const int i1 = s->dcf_pairs[2 * q] - 1, i2 = s->dcf_pairs[2 * q + 1] - 1;
        const double *F = &s->dcf_f[((size_t)irep * ndcf + q) * 3];
        for (int k = 0; k < 3; ++k) {
            forces[3 * i1 + k] = forces[3 * i1 + k] + F[k];
            forces[3 * i2 + k] = forces[3 * i2 + k] - F[k];
        }
    }
    for (int q = 0; q < (int)s->fr_pairs.size() / 2; ++q) {
        for (int t = 0; t < 2; ++t) {
            const int i = s->fr_pairs[2 * q + t] - 1;
            double p[3], v[3];
            for (int k = 0; k < 3; ++k) p[k] = s->fr_init[6 * q + 3 * t + k] + s->fr_velo[6 * q + 3 * t + k] * (double)istep;
            pbc_vec_d(s, p, &R.xyz[3 * i], v);
            for (int k = 0; k < 3; ++k) forces[3 * i + k] = forces[3 * i + k] + s->fr_k[2 * q + t] * v[k];
        }
    }
    if (s->rg_pott > 0) {
        double cm[3] = {0.0, 0.0, 0.0}, s2 = 0.0;
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) cm[k] += R.xyz[3 * i + k];
        for (int k = 0; k < 3; ++k) cm[k] /= (double)n;
        for (int i = 0; i < n; ++i) {
            double v[3] = {R.xyz[3 * i] - cm[0], R.xyz[3 * i + 1] - cm[1], R.xyz[3 * i + 2] - cm[2]};
            s2 += dot(v, v);
        }
        const double rg = sqrt(s2 / (double)n), r0 = s->rg0[irep];
        if (!(s->rg_pott == 2 && rg <= r0)) {
            const double factor = -s->rg_k * (rg - r0) / (rg * n);
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) forces[3 * i + k] = forces[3 * i + k] + factor * (R.xyz[3 * i + k] - cm[k]);
        }
    }
    for (int q = 0; q < (int)s->rest_id.size() / 3; ++q) {
        const int i = s->rest_id[3 * q] - 1, j = s->rest_id[3 * q + 1] - 1, type = s->rest_id[3 * q + 2];
        double v[3];
        pbc_vec_d(s, &R.xyz[3 * i], &R.xyz[3 * j], v);
        const double r = norm2(v);
        const double *pp = &s->rest_para[4 * q];
        if (r >= pp[3]) continue;
        const double th = tanh((r - pp[1]) / pp[2]);
        const double coef = 0.5 * pp[0] / pp[2] * (1.0 - th * th) / r;
        for (int k = 0; k < 3; ++k) {
            forces[3 * i + k] = forces[3 * i + k] - coef * v[k];
            if (type == 1) forces[3 * j + k] = forces[3 * j + k] + coef * v[k];
        }
    }
}

/* force.F90:1-77 : all terms.  Per-thread private buffers summed at the end as
 * force.F90:66-69 does.  istep: the reference's step number for the
 * time-dependent traps (the step being taken, or the steps taken outside
 * the MD loop). */
static void force_impl(or_system *s, int irep, double *forces, int only_term, int64_t istep) {
    Rep &R = s->rep[irep];
    const int n = s->nmp;
    const int nt = nthreads();
    std::vector<double> ft((size_t)nt * 3 * n, 0.0);
    const int nbond = (int)s->bond_mp.size() / 2, nangl = (int)s->angl_mp.size() / 3, ndih = (int)s->dih_mp.size() / 4;
    const int nwca = (int)R.wca_mp.size() / 2, nele = (int)R.ele_mp.size() / 2, nbp = (int)R.bp_mp.size() / 7;
    const bool triplet = s->p.bp_model == 4 || s->p.bp_model == 5;
    const double tK = R.tempK;
    R.ene_bp.assign(nbp, 0.0);
    R.bp_status.assign(nbp, 0);
#pragma omp parallel num_threads(nt)
    {
        int tn = 0, T = 1;
#ifdef _OPENMP
        tn = omp_get_thread_num();
        T = omp_get_num_threads();
#endif
        double *F = &ft[(size_t)tn * 3 * n];
        auto range = [&](int N, int &lo, int &hi) {
            int chunk = (N + T - 1) / T;
            lo = std::min(N, tn * chunk);
            hi = std::min(N, lo + chunk);
        };
        int lo, hi;
        if (only_term == 0 || only_term == 1) { range(nbond, lo, hi); force_bond(s, irep, F, lo, hi); }
        if (only_term == 0 || only_term == 2) {
            range(nangl, lo, hi);
            if (s->p.angl_reb) force_angl_reb(s, irep, F, lo, hi);
            else force_angl(s, irep, F, lo, hi);
        }
        if ((only_term == 0 || only_term == 3) && s->p.dih_type != 0) { range(ndih, lo, hi); force_dih(s, irep, F, lo, hi); }
        if ((only_term == 0 || only_term == 4) && !s->mc_now) {
            range(nbp, lo, hi);
            for (int k = lo; k < hi; ++k) {
                if (!R.bp_status_MC[k]) continue;
                double e;
                if (bp_one(s, irep, k, tK, F, &e)) {
                    R.ene_bp[k] = e;
                    R.bp_status[k] = 1;
                }
            }
        }
        if (only_term == 0 || only_term == 5) { range(nwca, lo, hi); force_wca(s, irep, F, lo, hi); }
        if ((only_term == 0 || only_term == 6) && s->p.flg_ele) { range(nele, lo, hi); force_ele(s, irep, F, lo, hi); }
    }
    (void)triplet;
    for (int i = 0; i < 3 * n; ++i) {
        double a = ft[i];
        for (int t = 1; t < nt; ++t) a += ft[(size_t)t * 3 * n + i];
        forces[i] = a;
    }
    if ((only_term == 0 || only_term == 4) && s->mc_now) bp_mc(s, irep, tK, forces);
    if (only_term == 0 || only_term == 4) s->flg_bp_energy = true;
    if (only_term == 0 || only_term == 7) force_bias(s, irep, forces, istep);
}

extern "C" void or_force(or_system *s, int32_t irep, double *forces) { force_impl(s, irep, forces, 0, s->istep); }
extern "C" void or_force_mc(or_system *s, int32_t irep, double *forces) {
    s->mc_now = true;
    force_impl(s, irep, forces, 0, s->istep);
    s->mc_now = false;
}
extern "C" int32_t or_get_mc_draws(const or_system *s, double *out, int32_t cap) {
    const int n = (int)s->mc_draws.size();
    for (int i = 0; i < std::min(n, cap); ++i) out[i] = s->mc_draws[i];
    return n;
}
extern "C" int32_t or_get_bp_status(const or_system *s, int32_t irep, uint8_t *out, int32_t cap) {
    const Rep &R = s->rep[irep];
    const int n = (int)R.bp_status.size();
    for (int i = 0; i < std::min(n, cap); ++i) out[i] = R.bp_status[i];
    return n;
}
extern "C" void or_force_term(or_system *s, int32_t irep, int32_t term, double *forces) {
    force_impl(s, irep, forces, term, s->istep);
}

/* ---------------------------------------------------------------- energies */
namespace {

/* energy_bp.F90 mp_angle / mp_dihedral */
double mp_angle(const or_system *s, int irep, int a, int b, int c) {
    double v12[3], v32[3];
    pbc_vec_d(s, X(s, irep, a), X(s, irep, b), v12);
    pbc_vec_d(s, X(s, irep, c), X(s, irep, b), v32);
    double co = dot(v32, v12) / sqrt(dot(v12, v12) * dot(v32, v32));
    if (co > 1.0) co = 1.0;
    else if (co < -1.0) co = -1.0;
    return acos(co);
}
double mp_dihedral(const or_system *s, int irep, int a, int b, int c, int d) {
    double v12[3], v32[3], v34[3], m[3], n[3];
    pbc_vec_d(s, X(s, irep, a), X(s, irep, b), v12);
    pbc_vec_d(s, X(s, irep, c), X(s, irep, b), v32);
    pbc_vec_d(s, X(s, irep, c), X(s, irep, d), v34);
    cross(v12, v32, m);
    cross(v32, v34, n);
    return atan2(dot(v12, n) * norm2(v32), dot(m, n));
}

} // namespace

/* energy_sumup.F90:1-56 with energy_{bond,angl,angl_ReB,dih_cos,dih_exp,bp,bp_triplet,wca,ele_DH}.F90 */
extern "C" void or_energy_sumup(or_system *s, int32_t irep, double tempK_in, double *E) {
    Rep &R = s->rep[irep];
    const or_params &p = s->p;
    for (int k = 0; k <= 10; ++k) E[k] = 0.0;
    /* energy_bond.F90:17-28 */
    for (size_t ib = 0; ib < s->bond_mp.size() / 2; ++ib) {
        double v[3];
        pbc_vec_d(s, X(s, irep, s->bond_mp[2 * ib]), X(s, irep, s->bond_mp[2 * ib + 1]), v);
        double d = norm2(v);
        E[1] = E[1] + 0.5 * p.bond_k * ((d - p.bond_r0) * (d - p.bond_r0));
    }
    /* energy_angl.F90:18-41 / energy_angl_ReB.F90 */
    const double co0 = cos(p.angl_t0);
    for (size_t ia = 0; ia < s->angl_mp.size() / 3; ++ia) {
        double v12[3], v32[3];
        pbc_vec_d(s, X(s, irep, s->angl_mp[3 * ia]), X(s, irep, s->angl_mp[3 * ia + 1]), v12);
        pbc_vec_d(s, X(s, irep, s->angl_mp[3 * ia + 2]), X(s, irep, s->angl_mp[3 * ia + 1]), v32);
        double t = dot(v32, v12) / sqrt(dot(v12, v12) * dot(v32, v32));
        if (p.angl_reb) {
            E[2] = E[2] + 0.5 * p.angl_k * ((t - co0) * (t - co0)) / (1.0 - t * t);
        } else {
            if (t > 1.0) t = 1.0;
            else if (t < -1.0) t = -1.0;
            t = acos(t);
            E[2] = E[2] + 0.5 * p.angl_k * ((t - p.angl_t0) * (t - p.angl_t0));
        }
    }
    /* energy_dih_cos.F90:18-39 / energy_dih_exp.F90 */
    if (p.dih_type != 0) {
        for (size_t id = 0; id < s->dih_mp.size() / 4; ++id) {
            const int *q = &s->dih_mp[4 * id];
            double v12[3], v23[3], v34[3], c1[3], c2[3];
            pbc_vec_d(s, X(s, irep, q[1]), X(s, irep, q[0]), v12);
            pbc_vec_d(s, X(s, irep, q[2]), X(s, irep, q[1]), v23);
            pbc_vec_d(s, X(s, irep, q[3]), X(s, irep, q[2]), v34);
            cross(v12, v23, c1);
            cross(v23, v34, c2);
            double dih = atan2(norm2(v23) * dot(v12, c2), dot(c1, c2));
            if (p.dih_type == 1)
                E[3] = E[3] + p.dih_k * (1.0 + cos(dih + p.dih_p0));
            else
                E[3] = E[3] - p.dih_k * exp((-0.5 * p.dih_w) * ((dih - p.dih_p0) * (dih - p.dih_p0)));
        }
    }
    /* energy_bp.F90 / energy_bp_triplet.F90: cached from the last force call when
     * flg_bp_energy is set, else recomputed */
    const int nbp = (int)R.bp_mp.size() / 7;
    const bool triplet = p.bp_model == 4 || p.bp_model == 5;
    if (!s->flg_bp_energy) {
        R.ene_bp.assign(nbp, 0.0);
        R.bp_status.assign(nbp, 0);
        double tK = (p.temp_independent == 0) ? tempK_in : 0.0;
        for (int k = 0; k < nbp; ++k) {
            if (!R.bp_status_MC[k]) continue;
            const int *rec = &R.bp_mp[7 * k];
            const BPP &b = s->bpp[rec[6]];
            double dG = 0.0;
            if (triplet) {
                dG = R.bp_coef[2 * k] - tK * R.bp_coef[2 * k + 1];
                if (dG >= 0.0) continue;
            }
            double v[3];
            pbc_vec_d(s, X(s, irep, rec[0]), X(s, irep, rec[1]), v);
            double d = norm2(v) - b.bond_r;
            if (fabs(d) > b.cutoff_ddist) continue;
            double u = b.bond_k * (d * d), th;
            th = mp_angle(s, irep, rec[0], rec[1], rec[3]);
            u = u + b.angl_k1 * ((th - b.angl_theta1) * (th - b.angl_theta1));
            th = mp_angle(s, irep, rec[2], rec[0], rec[1]);
            u = u + b.angl_k2 * ((th - b.angl_theta2) * (th - b.angl_theta2));
            th = mp_angle(s, irep, rec[0], rec[1], rec[5]);
            u = u + b.angl_k3 * ((th - b.angl_theta3) * (th - b.angl_theta3));
            th = mp_angle(s, irep, rec[4], rec[0], rec[1]);
            u = u + b.angl_k4 * ((th - b.angl_theta4) * (th - b.angl_theta4));
            double ph = mp_dihedral(s, irep, rec[2], rec[0], rec[1], rec[3]);
            u = u + b.dihd_k1 * (1.0 + cos(ph + b.dihd_phi1));
            ph = mp_dihedral(s, irep, rec[4], rec[0], rec[1], rec[5]);
            u = u + b.dihd_k2 * (1.0 + cos(ph + b.dihd_phi2));
            u = triplet ? b.U0 * dG * exp(-u) : b.U0 * exp(-u);
            if (u <= p.bp_cutoff_energy) {
                R.ene_bp[k] = u;
                R.bp_status[k] = 1;
            }
        }
    }
    for (int k = 0; k < nbp; ++k) E[4] += R.ene_bp[k];
    /* energy_wca.F90:19-33 */
    for (size_t k = 0; k < R.wca_mp.size() / 2; ++k) {
        double v[3];
        pbc_vec_d(s, X(s, irep, R.wca_mp[2 * k]), X(s, irep, R.wca_mp[2 * k + 1]), v);
        double d = norm2(v);
        if (d >= p.wca_sigma) continue;
        d = p.wca_sigma / d;
        double d6 = d * d * d * d * d * d;
        E[5] = E[5] + p.wca_eps * (d6 * d6 - 2.0 * d6 + 1.0);
    }
    /* energy_ele_DH.F90:20-37 */
    if (p.flg_ele) {
        const double rcdist = 1.0 / R.lambdaD;
        for (size_t k = 0; k < R.ele_mp.size() / 2; ++k) {
            double v[3];
            pbc_vec_d(s, X(s, irep, R.ele_mp[2 * k]), X(s, irep, R.ele_mp[2 * k + 1]), v);
            double dist = norm2(v);
            if (dist > R.ele_cutoff) continue;
            if (p.temp_independent == 0) {
                E[6] = E[6] + R.ele_coef / dist * exp(-dist * rcdist);
            } else {
                double rk = dist * rcdist;
                E[6] = E[6] + R.ele_coef / dist * exp(-rk) * (-(1.0 + 0.5 * rk) * R.diele_dTcoef);
            }
        }
    }
    /* energy_stage.F90, energy_tweezers.F90, energy_rg.F90, energy_restraint.F90 */
    if (s->stage) {
        const double eps4 = 4 * s->stage_eps;
        for (int i = 0; i < s->nmp; ++i) {
            const double z = s->stage_sigma / R.xyz[3 * i + 2];
            const double z2 = z * z, z6 = z2 * z2 * z2;
            E[7] = E[7] + eps4 * (z6 * z6 - z6);
        }
    }
    const int ndcf = (int)s->dcf_pairs.size() / 2;
    for (int q = 0; q < ndcf; ++q) {
        double v[3];
        pbc_vec_d(s, X(s, irep, s->dcf_pairs[2 * q]), X(s, irep, s->dcf_pairs[2 * q + 1]), v);
        E[8] = E[8] - dot(v, &s->dcf_f[((size_t)irep * ndcf + q) * 3]);
    }
    if (s->rg_pott > 0) {
        const double rg = or_rg(s, irep), r0 = s->rg0[irep];
        E[9] = (s->rg_pott == 2 && rg <= r0) ? 0.0 : 0.5 * s->rg_k * (rg - r0) * (rg - r0);
    }
    for (int q = 0; q < (int)s->rest_id.size() / 3; ++q) {
        double v[3];
        pbc_vec_d(s, X(s, irep, s->rest_id[3 * q]), X(s, irep, s->rest_id[3 * q + 1]), v);
        const double r = norm2(v);
        const double *pp = &s->rest_para[4 * q];
        if (r >= pp[3]) continue;
        E[10] = E[10] - 0.5 * pp[0] * (1.0 - tanh((r - pp[1]) / pp[2]));
    }
    double tot = 0.0;
    for (int k = 1; k <= 10; ++k) tot += E[k];
    E[0] = tot;
}

extern "C" void or_set_stage(or_system *s, double sigma, double eps) {
    s->stage = sigma > 0.0;
    s->stage_sigma = sigma;
    s->stage_eps = eps;
}
extern "C" void or_set_rg_bias(or_system *s, int32_t pott, double k, const double *rg0) {
    s->rg_pott = pott;
    s->rg_k = k;
    s->rg0.assign(rg0, rg0 + s->nrep);
}
extern "C" void or_set_restraints(or_system *s, int32_t n, const int32_t *ids3, const double *para4) {
    s->rest_id.assign(ids3, ids3 + 3 * n);
    s->rest_para.assign(para4, para4 + 4 * n);
}
extern "C" void or_set_tweezers(or_system *s, int32_t ndcf, const int32_t *dcf_pairs, const double *dcf_f, int32_t nfr,
                                const int32_t *fr_pairs, const double *fr_k, const double *fr_init, const double *fr_velo) {
    s->dcf_pairs.assign(dcf_pairs, dcf_pairs + 2 * ndcf);
    s->dcf_f.assign(dcf_f, dcf_f + (size_t)3 * ndcf * s->nrep);
    s->fr_pairs.assign(fr_pairs, fr_pairs + 2 * nfr);
    s->fr_k.assign(fr_k, fr_k + 2 * nfr);
    s->fr_init.assign(fr_init, fr_init + 6 * nfr);
    s->fr_velo.assign(fr_velo, fr_velo + 6 * nfr);
}

extern "C" void or_set_bp_energy_flag(or_system *s, int32_t f) { s->flg_bp_energy = f != 0; }
extern "C" int32_t or_get_bp_state(const or_system *s, int32_t irep, double *ene, uint8_t *st, int32_t cap) {
    const Rep &R = s->rep[irep];
    int n = (int)R.ene_bp.size(), m = std::min(n, cap);
    if (ene) memcpy(ene, R.ene_bp.data(), sizeof(double) * m);
    if (st) memcpy(st, R.bp_status.data(), m);
    return n;
}

/* energy_kinetic.F90:15-29 */
extern "C" double or_energy_kinetic(const or_system *s, int32_t irep) {
    const Rep &R = s->rep[irep];
    double e = 0.0;
    for (int i = 0; i < s->nmp; ++i) e = e + s->mass[i] * dot(&R.velos[3 * i], &R.velos[3 * i]);
    return 0.5 * e;
}

/* energy_rg.F90:17-26 (unweighted radius of gyration) */
extern "C" double or_rg(const or_system *s, int32_t irep) {
    const Rep &R = s->rep[irep];
    double cm[3] = {0, 0, 0};
    for (int i = 0; i < s->nmp; ++i)
        for (int k = 0; k < 3; ++k) cm[k] += R.xyz[3 * i + k];
    for (int k = 0; k < 3; ++k) cm[k] /= (double)s->nmp;
    double s2 = 0.0;
    for (int i = 0; i < s->nmp; ++i) {
        double v[3] = {R.xyz[3 * i] - cm[0], R.xyz[3 * i + 1] - cm[1], R.xyz[3 * i + 2] - cm[2]};
        s2 = s2 + dot(v, v);
    }
    return sqrt(s2 / (double)s->nmp);
}

/* -------------------------------------------------------------------- RNG */
/* mt_stream.F90:419-444 mt_init_by_scalar, :510-548 mt_genrand_int32 (tempered) */
extern "C" or_mt *or_mt_create(int32_t seed) {
    or_mt *m = new or_mt();
    uint32_t js = (uint32_t)seed;
    for (int i = 0; i < 624; ++i) {
        m->st[i] = js;
        js = 1812433253u * (js ^ (js >> 30)) + (uint32_t)i + 1u;
    }
    m->i = 624;
    m->stored = false;
    m->stored_value = 0.0;
    return m;
}
extern "C" void or_mt_destroy(or_mt *m) { delete m; }
extern "C" uint32_t or_mt_int32(or_mt *m) {
    const uint32_t UM = 0x80000000u, LM = 0x7fffffffu, A = 0x9908b0dfu;
    if (m->i >= 624) {
        int k;
        for (k = 0; k < 624 - 397; ++k) {
            uint32_t y = (m->st[k] & UM) | (m->st[k + 1] & LM);
            m->st[k] = m->st[k + 397] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
        }
        for (; k < 623; ++k) {
            uint32_t y = (m->st[k] & UM) | (m->st[k + 1] & LM);
            m->st[k] = m->st[k + 397 - 624] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
        }
        uint32_t y = (m->st[623] & UM) | (m->st[0] & LM);
        m->st[623] = m->st[396] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
        m->i = 0;
    }
    uint32_t y = m->st[m->i++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}
/* mt_stream.F90:708-727 genrand_double1: [0,1], 53-bit */
extern "C" double or_mt_double1(or_mt *m) {
    uint32_t ia = or_mt_int32(m) >> 5, ib = or_mt_int32(m) >> 6;
    return ((double)ia * 67108864.0 + (double)ib) * (1.0 / 9007199254740991.0);
}
/* mt_stream.F90:750-769 genrand_double3: (0,1), 52-bit */
extern "C" double or_mt_double3(or_mt *m) {
    uint32_t ia = or_mt_int32(m) >> 6, ib = or_mt_int32(m) >> 6;
    return ((double)ia * 67108864.0 + (double)ib + 0.5) * (1.0 / 4503599627370496.0);
}
/* rnd_boxmuller.F90:1-49 (polar method, one saved spare) */
static double boxmuller_draw(or_mt *m, bool &stored, double &stored_value) {
    if (!stored) {
        stored = true;
        double vx, vy, r2;
        for (;;) {
            vx = 2.0 * or_mt_double1(m) - 1.0;
            vy = 2.0 * or_mt_double1(m) - 1.0;
            r2 = vx * vx + vy * vy;
            if (r2 < 1.0 && r2 > 0.0) break;
        }
        double rf = sqrt(-2.0 * log(r2) / r2);
        stored_value = vx * rf;
        return vy * rf;
    }
    stored = false;
    return stored_value;
}
extern "C" double or_mt_boxmuller(or_mt *m) { return boxmuller_draw(m, m->stored, m->stored_value); }

/* ---------------------------------------------- MT19937 jump-ahead streams
 * mt_stream.F90:580-706 (mt_create_stream, mt_jumpahead) with f_get_coeff.F90
 * and gf2xe.F90: the state that is J = id * 2^jp outputs ahead is p(B) v,
 * where v is the state vector (624 words, pointer at 624), B the one-word
 * transition (mt_matvec) and p(x) = x^J mod f(x), f the characteristic
 * polynomial of MT19937 in closed form from (n, m, r, w, a) (f_get_coeff.F90:
 * 17-41).  The polynomial method is Haramoto, Matsumoto, Nishimura, Panneton
 * and L'Ecuyer, "Efficient jump ahead for F2-linear random number
 * generators", INFORMS J. Computing 20 (2008).  Polynomials over GF(2) are
 * bit vectors of 64-bit words, bit k the coefficient of x^k. */
namespace {
using Gf2 = std::vector<uint64_t>;

int gf2_deg(const Gf2 &a) {
    for (int w = (int)a.size() - 1; w >= 0; --w)
        if (a[w]) return 64 * w + 63 - __builtin_clzll(a[w]);
    return -1;
}
void gf2_trim(Gf2 &a) {
    while (!a.empty() && a.back() == 0) a.pop_back();
}
void gf2_set(Gf2 &a, int k) {
    if ((int)a.size() <= k / 64) a.resize(k / 64 + 1, 0);
    a[k / 64] ^= 1ull << (k % 64);
}
void gf2_add(Gf2 &a, const Gf2 &b) {
    if (a.size() < b.size()) a.resize(b.size(), 0);
    for (size_t i = 0; i < b.size(); ++i) a[i] ^= b[i];
    gf2_trim(a);
}
/* carry-less product of two words: (hi, lo) */
inline void clmul64(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
    uint64_t h = 0, l = 0;
    for (int i = 0; i < 64; ++i)
        if ((b >> i) & 1ull) {
            l ^= a << i;
            if (i) h ^= a >> (64 - i);
        }
    hi = h;
    lo = l;
}
Gf2 gf2_mul(const Gf2 &a, const Gf2 &b) {
    if (a.empty() || b.empty()) return {};
    Gf2 c(a.size() + b.size(), 0);
    for (size_t i = 0; i < a.size(); ++i) {
        if (!a[i]) continue;
        for (size_t j = 0; j < b.size(); ++j) {
            if (!b[j]) continue;
            uint64_t hi, lo;
            clmul64(a[i], b[j], hi, lo);
            c[i + j] ^= lo;
            c[i + j + 1] ^= hi;
        }
    }
    gf2_trim(c);
    return c;
}
Gf2 gf2_sqr(const Gf2 &a) {
    Gf2 c(2 * a.size(), 0);
    for (size_t i = 0; i < a.size(); ++i)
        for (int k = 0; k < 64; ++k)
            if ((a[i] >> k) & 1ull) gf2_set(c, (int)(128 * i) + 2 * k);
    gf2_trim(c);
    return c;
}
/* a mod f (long division, bit by bit from the top) */
void gf2_mod(Gf2 &a, const Gf2 &f, int df) {
    for (int d = gf2_deg(a); d >= df; d = gf2_deg(a)) {
        const int sh = d - df, ws = sh / 64, bs = sh % 64;
        for (size_t i = 0; i < f.size(); ++i) {
            if (!f[i]) continue;
            a[i + ws] ^= f[i] << bs;
            if (bs && i + ws + 1 < a.size()) a[i + ws + 1] ^= f[i] >> (64 - bs);
        }
        gf2_trim(a);
    }
}
Gf2 gf2_pow(const Gf2 &a, int e) {
    Gf2 r{1};
    for (int k = 0; k < e; ++k) r = gf2_mul(r, a);
    return r;
}
/* f_get_coeff.F90:17-41: the characteristic polynomial of MT19937 */
const Gf2 &mt_charpoly() {
    static Gf2 ff;
    if (!ff.empty()) return ff;
    const int nn = 624, mm = 397, rr = 31, ww = 32;
    const uint32_t avec = 0x9908b0dfu;
    Gf2 af, bf;
    gf2_set(af, nn);
    gf2_set(af, mm);
    gf2_set(bf, nn - 1);
    gf2_set(bf, mm - 1);
    const Gf2 f1 = gf2_pow(af, ww - rr);
    ff = gf2_mul(f1, gf2_pow(bf, rr));
    for (int i = 0; i < rr; ++i)
        if ((avec >> (i % ww)) & 1u) gf2_add(ff, gf2_mul(gf2_pow(bf, rr - 1 - i), f1));
    for (int i = rr; i < ww; ++i)
        if ((avec >> (i % ww)) & 1u) gf2_add(ff, gf2_pow(af, ww - 1 - i));
    return ff;
}
/* x^(id * 2^jp) mod f, cached by (jp, id) */
Gf2 mt_jump_poly(int jp, int id) {
    static std::map<std::pair<int, int>, Gf2> cache;
    static std::map<int, Gf2> base;
    const auto key = std::make_pair(jp, id);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const Gf2 &f = mt_charpoly();
    const int df = gf2_deg(f);
    auto bt = base.find(jp);
    if (bt == base.end()) {
        Gf2 p;
        gf2_set(p, 1); /* x */
        for (int k = 0; k < jp; ++k) {
            p = gf2_sqr(p);
            gf2_mod(p, f, df);
        }
        bt = base.emplace(jp, p).first;
    }
    Gf2 r{1};
    for (int k = 0; k < id; ++k) {
        r = gf2_mul(r, bt->second);
        gf2_mod(r, f, df);
    }
    cache.emplace(key, r);
    return r;
}
/* mt_stream.F90:551-578 mt_matvec: w = B v */
void mt_matvec(const uint32_t *v, uint32_t *w) {
    const uint32_t UM = 0x80000000u, LM = 0x7fffffffu, A = 0x9908b0dfu;
    w[0] = v[1] & UM;
    for (int k = 1; k < 623; ++k) w[k] = v[k + 1];
    const uint32_t is = (v[0] & UM) | (v[1] & LM);
    w[623] = v[397] ^ (is >> 1) ^ ((is & 1u) ? A : 0u);
}
} // namespace

/* mt_create_stream: `that` = `base` jumped id * 2^jp outputs ahead (the
 * base's pointer is put at 624 first, as mt_jumpahead does) */
extern "C" void or_mt_jump(or_mt *base, int32_t jp, int32_t id, or_mt *that) {
    base->i = 624;
    const Gf2 p = mt_jump_poly(jp, id);
    const int np = gf2_deg(p) + 1;
    uint32_t v[624], w[624], t[624];
    memcpy(v, base->st, sizeof v);
    memcpy(w, v, sizeof w); /* the top coefficient is 1 */
    for (int i = np - 2; i >= 0; --i) {
        mt_matvec(w, t);
        if ((p[i / 64] >> (i % 64)) & 1ull)
            for (int k = 0; k < 624; ++k) w[k] = v[k] ^ t[k];
        else
            memcpy(w, t, sizeof w);
    }
    memcpy(that->st, w, sizeof w);
    that->i = 624;
    that->stored = false;
    that->stored_value = 0.0;
}

/* init_mts.F90:21-43: one base stream from rng_seed; replica irep (grep =
 * irep, 1-based) draws from the stream jumped (grep + id_offset) * 2^256
 * ahead, id_offset = 1 when the run is a replica run (stream 1 then serves
 * the exchanges, mts_rep). */
extern "C" void or_seed_streams(or_system *s, int32_t seed, int32_t replica_run) {
    or_mt *base = or_mt_create(seed);
    for (int r = 0; r < s->nrep; ++r) or_mt_jump(base, 256, r + 1 + (replica_run ? 1 : 0), &s->mts[r]);
    or_mt_destroy(base);
    s->spare_stored = false;
}

extern "C" void or_seed(or_system *s, int32_t seed) {
    /* Replica r draws from an MT stream initialised by seed + r: independent
     * streams without the jump-ahead.  or_seed_streams derives the streams
     * the reference uses (init_mts.F90:21-43). */
    for (int r = 0; r < s->nrep; ++r) {
        or_mt *m = or_mt_create(seed + r);
        s->mts[r] = *m;
        or_mt_destroy(m);
    }
    s->spare_stored = false;
}

/* ------------------------------------------------------------- time loop */
extern "C" void or_md_init(or_system *s) {
    std::vector<double> f(3 * (size_t)s->nmp);
    for (int r = 0; r < s->nrep; ++r) {
        or_neighbor_list(s, r);
        std::fill(s->rep[r].xyz_move.begin(), s->rep[r].xyz_move.end(), 0.0);
        /* job_md.F90:270-273,344-345: the set-up evaluation runs the base-pair
           Monte Carlo and its survivors are the first mask */
        if (s->p.nstep_bp_mc > 0) or_force_mc(s, r, f.data());
    }
    s->nrebuild = 0;
    s->istep = 0;
}

/* job_md.F90:214-238 initial velocities and accelerations */
extern "C" void or_init_velocities(or_system *s) {
    for (int r = 0; r < s->nrep; ++r) {
        Rep &R = s->rep[r];
        for (int i = 0; i < s->nmp; ++i) {
            double c1 = sqrt(R.tempK * BOLTZ_KCAL_MOL / s->mass[i]);
            for (int k = 0; k < 3; ++k) R.velos[3 * i + k] = c1 * boxmuller_draw(&s->mts[r], s->spare_stored, s->spare_value);
        }
        for (int i = 0; i < s->nmp; ++i)
            for (int k = 0; k < 3; ++k)
                R.accels[3 * i + k] = R.md_coef_rep[i] * boxmuller_draw(&s->mts[r], s->spare_stored, s->spare_value);
    }
}

extern "C" int64_t or_nrebuild(const or_system *s) { return s->nrebuild; }

/* job_md.F90:360-460 */
extern "C" int64_t or_run(or_system *s, int64_t nsteps, const double *noise) {
    const int n = s->nmp;
    std::vector<double> forces(3 * n), rnd(3 * n);
    int64_t before = s->nrebuild;
    for (int64_t istep = 0; istep < nsteps; ++istep) {
        /* job_md.F90:364-367: Monte Carlo every nstep_bp_mc steps (1-based step
           count), and after every neighbour-list rebuild (:392-394) */
        const int nmc = s->p.nstep_bp_mc;
        const bool mc_step = nmc > 0 && (s->istep + 1) % nmc == 0;
        for (int r = 0; r < s->nrep; ++r) {
            Rep &R = s->rep[r];
            s->mc_now = mc_step;
            double d2max = 0.0, d2max_2nd = 0.0;
            for (int i = 0; i < n; ++i) {
                double d2 = dot(&R.xyz_move[3 * i], &R.xyz_move[3 * i]);
                if (d2 > d2max) {
                    d2max_2nd = d2max;
                    d2max = d2;
                } else if (d2 > d2max_2nd) {
                    d2max_2nd = d2;
                }
            }
            if (sqrt(d2max) + sqrt(d2max_2nd) > s->p.nl_margin) {
                or_neighbor_list(s, r);
                std::fill(R.xyz_move.begin(), R.xyz_move.end(), 0.0);
                if (nmc > 0) s->mc_now = true;
            }
            force_impl(s, r, forces.data(), 0, s->istep + 1);
            s->mc_now = false;
            if (noise) {
                memcpy(rnd.data(), noise + ((size_t)istep * s->nrep + r) * 3 * n, sizeof(double) * 3 * n);
            } else {
                for (int i = 0; i < 3 * n; ++i) rnd[i] = boxmuller_draw(&s->mts[r], s->spare_stored, s->spare_value);
            }
            if (s->p.integrator == 1) {
#pragma omp parallel for schedule(static)
                for (int i = 0; i < n; ++i) {
                    for (int k = 0; k < 3; ++k) {
                        double ap = R.md_coef_rep[i] * rnd[3 * i + k];
                        R.velos[3 * i + k] = s->md_coef[3 * i + 0] * R.velos[3 * i + k] + s->md_coef[3 * i + 1] * forces[3 * i + k] +
                                             (R.accels[3 * i + k] + ap);
                        R.accels[3 * i + k] = ap;
                        double dx = s->md_coef[3 * i + 2] * R.velos[3 * i + k];
                        R.xyz[3 * i + k] = R.xyz[3 * i + k] + dx;
                        R.xyz_move[3 * i + k] = R.xyz_move[3 * i + k] + dx;
                    }
                }
            } else {
#pragma omp parallel for schedule(static)
                for (int i = 0; i < n; ++i) {
                    for (int k = 0; k < 3; ++k) {
                        double dx = s->md_coef[3 * i + 0] * forces[3 * i + k] + R.md_coef_rep[i] * rnd[3 * i + k];
                        R.xyz[3 * i + k] = R.xyz[3 * i + k] + dx;
                        R.xyz_move[3 * i + k] = R.xyz_move[3 * i + k] + dx;
                    }
                }
            }
        }
        s->istep++;
    }
    return s->nrebuild - before;
}
