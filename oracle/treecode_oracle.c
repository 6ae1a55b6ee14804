/*
 * TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
 * Plain-C FP64 restatement of the reference's CPU tree-code path; see
 * treecode_oracle.h for the contract.  Reference paths are relative to the
 * reference project.  Operation order follows the reference expression by
 * expression so that, compiled with -ffp-contract=off, results are bitwise
 * identical to the compiled reference on the same inputs.
 */
#include "treecode_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* kernel radial factors                                               */
/* ------------------------------------------------------------------ */

/* t-SNE: nBodySolverFMM_SYM_MORTON.h:624-636 (D1 = rS^-2, D2 = -4 rS^-3,
 * D3 = 24 rS^-4).  Gravity: F(R) = R g(s), g = -(s + eps^2)^-3/2,
 * D1 = g, D2 = 2g', D3 = 4g''; pair term t = -(s + eps^2)^-1/2.          */
typedef struct { double D1, D2, D3, t; } derivs;

static inline derivs tsne_derivs(double sq_r)
{
    derivs d;
    double rS = 1.0 + sq_r;
    double inv = 1.0 / rS;
    double inv2 = inv * inv;
    double inv3 = inv2 * inv;
    double inv4 = inv3 * inv;
    d.D1 = inv2;
    d.D2 = -4.0 * inv3;
    d.D3 = 24.0 * inv4;
    d.t = rS; /* callers divide by rS as the reference does */
    return d;
}

static inline derivs grav_derivs(double s, double eps2)
{
    derivs d;
    double u = s + eps2;
    double iu = 1.0 / u;
    double isq = 1.0 / sqrt(u);
    double g = -isq * iu;
    d.D1 = g;
    d.D2 = -3.0 * g * iu;
    d.D3 = -5.0 * d.D2 * iu;
    d.t = -isq;
    return d;
}

/* C1 from a source of mass MB0 and second moment MB2 at offset R
 * (nBodySolverFMM_SYM_MORTON.h:638-655).                                   */
static inline void far_c1(double Rx, double Ry, double MB0, const double* MB2,
                          double D1, double D2, double D3, double* out)
{
    double inv = 1.0 / MB0;
    double T00 = inv * MB2[0], T01 = inv * MB2[1], T10 = inv * MB2[2], T11 = inv * MB2[3];
    double S1 = T00 + T11;
    double S2 = (Rx * Rx * T00) + (Rx * Ry * T01) + (Ry * Rx * T10) + (Ry * Ry * T11);
    double S30 = Rx * T00 + Ry * T01;
    double S31 = Rx * T10 + Ry * T11;
    out[0] = MB0 * (Rx * (D1 + 0.5 * (S1)*D2 + 0.5 * (S2)*D3) + (S30)*D2);
    out[1] = MB0 * (Ry * (D1 + 0.5 * (S1)*D2 + 0.5 * (S2)*D3) + (S31)*D2);
}

/* C2/C3 block (nBodySolverFMM_SYM_MORTON.h:657-697): C2 = MA0*(MB0*(...)).
 * has_mb selects the P2L form (:764-804) that has no MB0 factor.            */
static inline void c2c3(double Rx, double Ry, double MA0, double MB0, int has_mb,
                        double D1, double D2, double D3, double* C2, double* C3)
{
    double r[2] = {Rx, Ry};
    double e2[4], e3[8];
    e2[0] = (D1 + Rx * Rx * D2);
    e2[1] = (Rx * Ry * D2);
    e2[2] = (Ry * Rx * D2);
    e2[3] = (D1 + Ry * Ry * D2);
    e3[0] = ((Rx + Rx + Rx) * D2 + Rx * Rx * Rx * D3);
    e3[1] = ((Ry)*D2 + Rx * Rx * Ry * D3);
    e3[2] = ((Ry)*D2 + Rx * Ry * Rx * D3);
    e3[3] = ((Rx)*D2 + Rx * Ry * Ry * D3);
    e3[4] = ((Ry)*D2 + Ry * Rx * Rx * D3);
    e3[5] = ((Rx)*D2 + Ry * Rx * Ry * D3);
    e3[6] = ((Rx)*D2 + Ry * Ry * Rx * D3);
    e3[7] = ((Ry + Ry + Ry) * D2 + Ry * Ry * Ry * D3);
    (void)r;
    for (int i = 0; i < 4; i++) C2[i] = has_mb ? MA0 * (MB0 * e2[i]) : MA0 * e2[i];
    for (int i = 0; i < 8; i++) C3[i] = has_mb ? MA0 * (MB0 * e3[i]) : MA0 * e3[i];
}

/* Gravity kernels use the same expression layout as the t-SNE kernels.
 * The gravity C2/C3 are built with (MA0*MB0) as one factor, matching the
 * reference-side gravity kernels in oracle/ref_harness.cpp.               */
static inline void c2c3_grav(double Rx, double Ry, double scale, double D1, double D2,
                             double D3, double* C2, double* C3)
{
    double r[2] = {Rx, Ry};
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            C2[i * 2 + j] = scale * ((i == j ? D1 : 0.0) + r[i] * r[j] * D2);
            for (int k = 0; k < 2; k++) {
                double d = ((i == j) ? r[k] : 0.0) + ((i == k) ? r[j] : 0.0) + ((j == k) ? r[i] : 0.0);
                C3[i * 4 + j * 2 + k] = scale * (d * D2 + r[i] * r[j] * r[k] * D3);
            }
        }
}

typedef struct {
    int kernel;
    double eps2;
    double theta;
    const double* pos;
    double* grad;
    orc_node* nodes;
    double total;
} sym_ctx;

/* TSNE_FMM_SYM_MORTON_NN_Kernel (:622-723) / gravity counterpart */
static void kernel_nn(sym_ctx* c, orc_node* A, orc_node* B)
{
    double Rx = A->com[0] - B->com[0];
    double Ry = A->com[1] - B->com[1];
    double sq = Rx * Rx + Ry * Ry;
    double C1[2], C2[4], C3[8];
    if (c->kernel == ORC_KERNEL_TSNE) {
        derivs d = tsne_derivs(sq);
        far_c1(Rx, Ry, B->m0, B->m2, d.D1, d.D2, d.D3, C1);
        c2c3(Rx, Ry, A->m0, B->m0, 1, d.D1, d.D2, d.D3, C2, C3);
        A->c1[0] += C1[0]; A->c1[1] += C1[1];
        for (int i = 0; i < 4; i++) A->c2[i] += C2[i];
        for (int i = 0; i < 8; i++) A->c3[i] += C3[i];
        far_c1(-Rx, -Ry, A->m0, A->m2, d.D1, d.D2, d.D3, C1);
        B->c1[0] += C1[0]; B->c1[1] += C1[1];
        for (int i = 0; i < 4; i++) B->c2[i] += C2[i];
        for (int i = 0; i < 8; i++) B->c3[i] += -C3[i];
        c->total += 2.0 * (A->m0 * B->m0) / d.t;
    } else {
        derivs d = grav_derivs(sq, c->eps2);
        far_c1(Rx, Ry, B->m0, B->m2, d.D1, d.D2, d.D3, C1);
        c2c3_grav(Rx, Ry, A->m0 * B->m0, d.D1, d.D2, d.D3, C2, C3);
        A->c1[0] += C1[0]; A->c1[1] += C1[1];
        for (int i = 0; i < 4; i++) A->c2[i] += C2[i];
        for (int i = 0; i < 8; i++) A->c3[i] += C3[i];
        far_c1(-Rx, -Ry, A->m0, A->m2, d.D1, d.D2, d.D3, C1);
        B->c1[0] += C1[0]; B->c1[1] += C1[1];
        for (int i = 0; i < 4; i++) B->c2[i] += C2[i];
        for (int i = 0; i < 8; i++) B->c3[i] += -C3[i];
        c->total += 2.0 * (A->m0 * B->m0) * d.t;
    }
}

/* TSNE_FMM_SYM_MORTON_PN_Kernel (:726-815) / gravity counterpart */
static void kernel_pn(sym_ctx* c, int64_t p, orc_node* B)
{
    const double* x = c->pos + 2 * p;
    double Rx = x[0] - B->com[0];
    double Ry = x[1] - B->com[1];
    double sq = Rx * Rx + Ry * Ry;
    double C1[2], C2[4], C3[8];
    derivs d = (c->kernel == ORC_KERNEL_TSNE) ? tsne_derivs(sq) : grav_derivs(sq, c->eps2);
    far_c1(Rx, Ry, B->m0, B->m2, d.D1, d.D2, d.D3, C1);
    c->grad[2 * p] += C1[0];
    c->grad[2 * p + 1] += C1[1];
    Rx = -Rx;
    Ry = -Ry;
    if (c->kernel == ORC_KERNEL_TSNE) {
        c2c3(Rx, Ry, B->m0, 1.0, 0, d.D1, d.D2, d.D3, C2, C3);
    } else {
        c2c3_grav(Rx, Ry, B->m0, d.D1, d.D2, d.D3, C2, C3);
    }
    B->c1[0] += (Rx * d.D1);
    B->c1[1] += (Ry * d.D1);
    for (int i = 0; i < 4; i++) B->c2[i] += C2[i];
    for (int i = 0; i < 8; i++) B->c3[i] += C3[i];
    if (c->kernel == ORC_KERNEL_TSNE)
        c->total += 2.0 * B->m0 / d.t;
    else
        c->total += 2.0 * B->m0 * d.t;
}

/* TSNE_FMM_SYM_MORTON_PP_Kernel (:818-836) / gravity counterpart */
static void kernel_pp(sym_ctx* c, int64_t a, int64_t b)
{
    const double* xa = c->pos + 2 * a;
    const double* xb = c->pos + 2 * b;
    double Rx = xa[0] - xb[0];
    double Ry = xa[1] - xb[1];
    double sq = Rx * Rx + Ry * Ry;
    if (c->kernel == ORC_KERNEL_TSNE) {
        double fd = 1.0 / (1.0 + sq);
        c->grad[2 * a] += fd * fd * Rx;
        c->grad[2 * a + 1] += fd * fd * Ry;
        c->grad[2 * b] += fd * fd * (-Rx);
        c->grad[2 * b + 1] += fd * fd * (-Ry);
        c->total += 2.0 * fd;
    } else {
        derivs d = grav_derivs(sq, c->eps2);
        c->grad[2 * a] += d.D1 * Rx;
        c->grad[2 * a + 1] += d.D1 * Ry;
        c->grad[2 * b] += d.D1 * (-Rx);
        c->grad[2 * b + 1] += d.D1 * (-Ry);
        c->total += 2.0 * d.t;
    }
}

/* ------------------------------------------------------------------ */
/* tree construction                                                   */
/* ------------------------------------------------------------------ */

uint32_t orc_get_depth(int max_children, int64_t n)
{
    /* N / max_children is integer division in the reference (int / int).   */
    const double circle_area = 3.141592653589793238462643383279502884 / 4.0;
    double depth_real = log((1.0 / circle_area) * (double)((int)n / max_children)) / log(4.0);
    return (uint32_t)ceil(depth_real);
}

int64_t orc_node_count(uint32_t depth)
{
    int64_t total = 0, s = 1;
    for (uint32_t l = 0; l <= depth; l++) {
        total += s;
        s *= 4;
    }
    return total;
}

static int64_t level_index(uint32_t l) { return (((int64_t)1 << (2 * l)) - 1) / 3; }

static inline uint32_t spread16(uint32_t x)
{
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

static inline double dmin(double a, double b) { return (b < a) ? b : a; }
static inline double dmax(double a, double b) { return (a < b) ? b : a; }

void orc_morton_codes(int64_t n, const double* pos, const double min_xy[2],
                      const double max_xy[2], uint32_t* codes)
{
    double nmx = -min_xy[0], nmy = -min_xy[1];
    double L = dmax(max_xy[0] + nmx, max_xy[1] + nmy); /* compMax (:84-85) */
    for (int64_t i = 0; i < n; i++) {
        double px = (pos[2 * i] + nmx) / (L);
        double py = (pos[2 * i + 1] + nmy) / (L);
        px = dmin(dmax(px * 65536.0, 0.0), 65535.0);
        py = dmin(dmax(py * 65536.0, 0.0), 65535.0);
        codes[i] = (spread16((uint32_t)py) << 1) | spread16((uint32_t)px);
    }
}

/* stable LSD counting sort on 8-bit digits (re-entrant; ties keep input order) */
void orc_sort_perm(int64_t n, const uint32_t* codes, int32_t* perm)
{
    int32_t* tmp = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    int32_t *src = perm, *dst = tmp;
    for (int64_t i = 0; i < n; i++) perm[i] = (int32_t)i;
    for (int shift = 0; shift < 32; shift += 8) {
        int64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (int64_t i = 0; i < n; i++) cnt[((codes[src[i]] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n; i++) dst[cnt[(codes[src[i]] >> shift) & 255u]++] = src[i];
        int32_t* t = src;
        src = dst;
        dst = t;
    }
    /* four passes: the result is back in perm */
    free(tmp);
}

void orc_build_tree(uint32_t depth, int64_t n, const double* pos, const double min_xy[2],
                    const double max_xy[2], orc_node* nodes)
{
    int64_t nn = orc_node_count(depth);
    memset(nodes, 0, (size_t)nn * sizeof(orc_node));
    double nmx = -min_xy[0], nmy = -min_xy[1];
    double L = dmax(max_xy[0] + nmx, max_xy[1] + nmy);
    uint32_t W = 1u << depth;
    double h = L / (double)W;
    int64_t base = level_index(depth);
    /* createLeafNodes (:328-379) */
    for (int64_t i = 0; i < n; i++) {
        double gx = (double)W * (pos[2 * i] + nmx) / (L);
        double gy = (double)W * (pos[2 * i + 1] + nmy) / (L);
        uint32_t ux = (uint32_t)gx, uy = (uint32_t)gy;
        if (ux > W - 1u) ux = W - 1u;
        if (uy > W - 1u) uy = W - 1u;
        orc_node* q = &nodes[base + ((spread16(uy) << 1) | spread16(ux))];
        if (q->count == 0u) {
            q->bb_c[0] = min_xy[0] + h * (double)ux + 0.5 * h;
            q->bb_c[1] = min_xy[1] + h * (double)uy + 0.5 * h;
            q->bb_len = h;
            q->first_part = (uint32_t)i;
        }
        q->count += 1u;
        q->com[0] += pos[2 * i];
        q->com[1] += pos[2 * i + 1];
    }
    for (int64_t k = base; k < base + ((int64_t)1 << (2 * depth)); k++) {
        orc_node* q = &nodes[k];
        if (q->count == 0u) continue;
        q->m0 = q->count;
        q->com[0] /= q->m0;
        q->com[1] /= q->m0;
        for (uint32_t p = q->first_part; p < q->first_part + q->count; p++) {
            double rx = pos[2 * p] - q->com[0];
            double ry = pos[2 * p + 1] - q->com[1];
            q->m2[0] += rx * rx;
            q->m2[1] += rx * ry;
            q->m2[2] += ry * rx;
            q->m2[3] += ry * ry;
        }
    }
    /* bottomUpNodeConstruction (:381-470) */
    static const double off[4][2] = {{0.5, 0.5}, {-0.5, 0.5}, {0.5, -0.5}, {-0.5, -0.5}};
    for (int l = (int)depth - 1; l >= 0; l--) {
        int64_t li = level_index((uint32_t)l), lc = level_index((uint32_t)l + 1);
        int64_t ls = (int64_t)1 << (2 * l);
        for (int64_t i = 0; i < ls; i++) {
            orc_node* q = &nodes[li + i];
            int64_t fc = lc + 4 * i;
            for (int j = 3; j >= 0; j--) {
                orc_node* ch = &nodes[fc + j];
                if (ch->count == 0u) continue;
                q->first_child = (uint32_t)fc;
                q->bb_c[0] = off[j][0] * ch->bb_len + ch->bb_c[0];
                q->bb_c[1] = off[j][1] * ch->bb_len + ch->bb_c[1];
                q->bb_len = 2.0 * ch->bb_len;
                q->first_part = ch->first_part;
                q->count += ch->count;
                q->com[0] += ch->m0 * ch->com[0];
                q->com[1] += ch->m0 * ch->com[1];
                q->m0 += ch->m0;
            }
            if (q->count == 0u) continue;
            q->com[0] /= q->m0;
            q->com[1] /= q->m0;
            for (int64_t c = q->first_child; c < (int64_t)q->first_child + 4; c++) {
                orc_node* ch = &nodes[c];
                if (ch->m0 == 0.0) continue;
                double rx = ch->com[0] - q->com[0];
                double ry = ch->com[1] - q->com[1];
                q->m2[0] += rx * rx;
                q->m2[1] += rx * ry;
                q->m2[2] += ry * rx;
                q->m2[3] += ry * ry;
                for (int t = 0; t < 4; t++) q->m2[t] += ch->m2[t];
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* symmetric dual-tree traversal                                       */
/* ------------------------------------------------------------------ */

/* traverse_SYM_PN (:272-313) */
static void trav_pn(sym_ctx* c, int64_t p, orc_node* B)
{
    const double* x = c->pos + 2 * p;
    double dx = x[0] - B->com[0], dy = x[1] - B->com[1];
    double dist = dx * dx + dy * dy;
    double thr = B->bb_len / c->theta;
    if (dist > thr * thr) {
        kernel_pn(c, p, B);
    } else if (B->first_child == 0) {
        for (int64_t q = B->first_part; q < (int64_t)B->first_part + B->count; q++)
            if (q != p) kernel_pp(c, p, q);
    } else {
        for (uint32_t k = B->first_child; k < B->first_child + 4; k++)
            if (c->nodes[k].count != 0) trav_pn(c, p, &c->nodes[k]);
    }
}

/* traverse_SYM_NN (:154-270).  Point identity uses the sorted index, which is
 * equivalent to the reference's ID check when IDs are unique.              */
static void trav_nn(sym_ctx* c, orc_node* A, orc_node* B)
{
    double dx = A->com[0] - B->com[0], dy = A->com[1] - B->com[1];
    double dist = dx * dx + dy * dy;
    double thr = (A->bb_len + B->bb_len) / c->theta;
    if (dist > thr * thr) {
        if (A->count != 0 && B->count != 0) kernel_nn(c, A, B);
    } else if (A->first_child == 0) {
        if (A == B) {
            for (int64_t i = A->first_part; i < (int64_t)A->first_part + A->count; i++)
                if (B->count != 0)
                    for (int64_t j = i; j < (int64_t)B->first_part + B->count; j++)
                        if (i != j) kernel_pp(c, i, j);
        } else {
            for (int64_t i = A->first_part; i < (int64_t)A->first_part + A->count; i++)
                if (B->count != 0) trav_pn(c, i, B);
        }
    } else if (B->first_child == 0) {
        if (A == B) {
            for (int64_t j = B->first_part; j < (int64_t)B->first_part + B->count; j++)
                if (A->count != 0)
                    for (int64_t i = j; i < (int64_t)A->first_part + A->count; i++)
                        if (i != j) kernel_pp(c, i, j);
        } else {
            for (int64_t j = B->first_part; j < (int64_t)B->first_part + B->count; j++)
                if (A->count != 0) trav_pn(c, j, A);
        }
    } else {
        for (uint32_t a = A->first_child; a < A->first_child + 4; a++) {
            uint32_t b0 = (A == B) ? a : B->first_child;
            for (uint32_t b = b0; b < B->first_child + 4; b++)
                if (c->nodes[a].count != 0 && c->nodes[b].count != 0)
                    trav_nn(c, &c->nodes[a], &c->nodes[b]);
        }
    }
}

/* einsum<Index<0>,Index<0,1>>(d, C2)_j = sum_i d_i C2_ij                   */
static inline void contract2(const double* d, const double* C2, double* out)
{
    out[0] = d[0] * C2[0] + d[1] * C2[2];
    out[1] = d[0] * C2[1] + d[1] * C2[3];
}
/* einsum<Index<0>,Index<0,1,2>>(d, C3)_jk = sum_i d_i C3_ijk               */
static inline void contract3(const double* d, const double* C3, double* out)
{
    for (int jk = 0; jk < 4; jk++) out[jk] = d[0] * C3[jk] + d[1] * C3[4 + jk];
}

/* applyForces (:482-536): L2L into non-empty children, L2P at leaves.      */
static void apply_forces(sym_ctx* c, orc_node* q)
{
    if (q->first_child != 0) {
        for (uint32_t k = q->first_child; k < q->first_child + 4; k++) {
            orc_node* ch = &c->nodes[k];
            if (ch->count == 0) continue;
            double inv = 1.0 / ch->m0;
            for (int i = 0; i < 4; i++) ch->c2[i] *= inv;
            for (int i = 0; i < 8; i++) ch->c3[i] *= inv;
            double d[2] = {ch->com[0] - q->com[0], ch->com[1] - q->com[1]};
            double e1[2], e3[4], e31[2], e2[4];
            contract2(d, q->c2, e1);
            contract3(d, q->c3, e3);
            contract2(d, e3, e31);
            for (int i = 0; i < 2; i++) ch->c1[i] += q->c1[i] + e1[i] + 0.5 * e31[i];
            for (int i = 0; i < 4; i++) e2[i] = q->c2[i] + e3[i];
            for (int i = 0; i < 4; i++) ch->c2[i] += e2[i];
            for (int i = 0; i < 8; i++) ch->c3[i] += q->c3[i];
            apply_forces(c, ch);
        }
    } else {
        for (int64_t p = q->first_part; p < (int64_t)q->first_part + q->count; p++) {
            double d[2] = {c->pos[2 * p] - q->com[0], c->pos[2 * p + 1] - q->com[1]};
            double e1[2], e3[4], e31[2];
            contract2(d, q->c2, e1);
            contract3(d, q->c3, e3);
            contract2(d, e3, e31);
            c->grad[2 * p] += q->c1[0] + e1[0] + 0.5 * e31[0];
            c->grad[2 * p + 1] += q->c1[1] + e1[1] + 0.5 * e31[1];
        }
    }
}

void orc_sym_fmm_solve(int kernel, double eps, uint32_t depth, double theta, int64_t n,
                       const double* pos, orc_node* nodes, double* grad, double* total)
{
    (void)depth;
    (void)n;
    sym_ctx c;
    c.kernel = kernel;
    c.eps2 = eps * eps;
    c.theta = theta;
    c.pos = pos;
    c.grad = grad;
    c.nodes = nodes;
    c.total = *total;
    trav_nn(&c, &nodes[0], &nodes[0]);
    double inv = 1.0 / nodes[0].m0;
    for (int i = 0; i < 4; i++) nodes[0].c2[i] *= inv;
    for (int i = 0; i < 8; i++) nodes[0].c3[i] *= inv;
    apply_forces(&c, &nodes[0]);
    *total = c.total;
}

/* ------------------------------------------------------------------ */
/* non-symmetric FMM_MORTON (nBodySolverFMM_MORTON.h)                  */
/* ------------------------------------------------------------------ */

/* the non-symmetric kernels' radial factors (:517-522): D1 = 1/(rS rS),
 * D2 = -4/(rS rS rS), D3 = 24/(rS rS rS rS) -- divided directly, which
 * rounds differently from the symmetric kernels' reciprocal powers          */
static inline derivs tsne_derivs_m(double sq_r)
{
    derivs d;
    double rS = 1.0 + sq_r;
    d.D1 = 1.0 / (rS * rS);
    d.D2 = -4.0 / (rS * rS * rS);
    d.D3 = 24.0 / (rS * rS * rS * rS);
    d.t = rS;
    return d;
}

/* TSNEFMM_MORTONNNKernel (:513-582) / gravity counterpart: the sink only;
 * C2 and C3 carry the source mass alone (no MA0).                          */
static void m_kernel_nn(sym_ctx* c, orc_node* A, orc_node* B)
{
    double Rx = A->com[0] - B->com[0];
    double Ry = A->com[1] - B->com[1];
    double sq = Rx * Rx + Ry * Ry;
    double C1[2], C2[4], C3[8];
    derivs d = (c->kernel == ORC_KERNEL_TSNE) ? tsne_derivs_m(sq) : grav_derivs(sq, c->eps2);
    if (c->kernel == ORC_KERNEL_TSNE)
        c->total += (A->m0 * B->m0) / d.t;
    else
        c->total += (A->m0 * B->m0) * d.t;
    far_c1(Rx, Ry, B->m0, B->m2, d.D1, d.D2, d.D3, C1);
    if (c->kernel == ORC_KERNEL_TSNE)
        c2c3(Rx, Ry, B->m0, 1.0, 0, d.D1, d.D2, d.D3, C2, C3);
    else
        c2c3_grav(Rx, Ry, B->m0, d.D1, d.D2, d.D3, C2, C3);
    A->c1[0] += C1[0]; A->c1[1] += C1[1];
    for (int i = 0; i < 4; i++) A->c2[i] += C2[i];
    for (int i = 0; i < 8; i++) A->c3[i] += C3[i];
}

/* TSNEFMM_MORTONPNKernel (:584-613): M2P into the sink point              */
static void m_kernel_pn(sym_ctx* c, int64_t p, orc_node* B)
{
    const double* x = c->pos + 2 * p;
    double Rx = x[0] - B->com[0];
    double Ry = x[1] - B->com[1];
    double sq = Rx * Rx + Ry * Ry;
    double C1[2];
    derivs d = (c->kernel == ORC_KERNEL_TSNE) ? tsne_derivs_m(sq) : grav_derivs(sq, c->eps2);
    if (c->kernel == ORC_KERNEL_TSNE)
        c->total += B->m0 / d.t;
    else
        c->total += B->m0 * d.t;
    far_c1(Rx, Ry, B->m0, B->m2, d.D1, d.D2, d.D3, C1);
    c->grad[2 * p] += C1[0];
    c->grad[2 * p + 1] += C1[1];
}

/* TSNEFMM_MORTONNPKernel (:615-673): P2L into the sink node (unit mass)   */
static void m_kernel_np(sym_ctx* c, orc_node* A, int64_t p)
{
    const double* x = c->pos + 2 * p;
    double Rx = A->com[0] - x[0];
    double Ry = A->com[1] - x[1];
    double sq = Rx * Rx + Ry * Ry;
    double C2[4], C3[8];
    derivs d = (c->kernel == ORC_KERNEL_TSNE) ? tsne_derivs_m(sq) : grav_derivs(sq, c->eps2);
    if (c->kernel == ORC_KERNEL_TSNE) {
        c->total += A->m0 / d.t;
        c2c3(Rx, Ry, 1.0, 1.0, 0, d.D1, d.D2, d.D3, C2, C3);
    } else {
        c->total += A->m0 * d.t;
        c2c3_grav(Rx, Ry, 1.0, d.D1, d.D2, d.D3, C2, C3);
    }
    A->c1[0] += (Rx * d.D1);
    A->c1[1] += (Ry * d.D1);
    for (int i = 0; i < 4; i++) A->c2[i] += C2[i];
    for (int i = 0; i < 8; i++) A->c3[i] += C3[i];
}

/* TSNEFMM_MORTONPPKernel (:675-683): the sink point only                  */
static void m_kernel_pp(sym_ctx* c, int64_t a, int64_t b)
{
    const double* xa = c->pos + 2 * a;
    const double* xb = c->pos + 2 * b;
    double Rx = xa[0] - xb[0];
    double Ry = xa[1] - xb[1];
    double sq = Rx * Rx + Ry * Ry;
    if (c->kernel == ORC_KERNEL_TSNE) {
        double fd = 1.0 / (1.0 + sq);
        c->total += fd;
        c->grad[2 * a] += fd * fd * Rx;
        c->grad[2 * a + 1] += fd * fd * Ry;
    } else {
        derivs d = grav_derivs(sq, c->eps2);
        c->total += d.t;
        c->grad[2 * a] += d.D1 * Rx;
        c->grad[2 * a + 1] += d.D1 * Ry;
    }
}

/* traverseBHMP (:199-232): point-node MAC L_B / |x - com_B| < theta        */
static void m_trav_bhmp(sym_ctx* c, int64_t p, orc_node* B)
{
    const double* x = c->pos + 2 * p;
    double dx = x[0] - B->com[0], dy = x[1] - B->com[1];
    double dist = sqrt(dx * dx + dy * dy);
    if (B->bb_len / dist < c->theta) {
        m_kernel_pn(c, p, B);
    } else if (B->first_child == 0) {
        for (int64_t q = B->first_part; q < (int64_t)B->first_part + B->count; q++)
            if (q != p) m_kernel_pp(c, p, q);
    } else {
        for (uint32_t k = B->first_child; k < B->first_child + 4; k++)
            if (c->nodes[k].count != 0) m_trav_bhmp(c, p, &c->nodes[k]);
    }
}

/* traverseBHRMP (:234-268): node-point MAC L_A / |com_A - x| < theta       */
static void m_trav_bhrmp(sym_ctx* c, orc_node* A, int64_t p)
{
    const double* x = c->pos + 2 * p;
    double dx = A->com[0] - x[0], dy = A->com[1] - x[1];
    double dist = sqrt(dx * dx + dy * dy);
    if (A->bb_len / dist < c->theta) {
        m_kernel_np(c, A, p);
    } else if (A->first_child == 0) {
        for (int64_t q = A->first_part; q < (int64_t)A->first_part + A->count; q++)
            if (q != p) m_kernel_pp(c, q, p);
    } else {
        for (uint32_t k = A->first_child; k < A->first_child + 4; k++)
            if (c->nodes[k].count != 0) m_trav_bhrmp(c, &c->nodes[k], p);
    }
}

/* traverseFMM (:148-197): ordered (sink, source) pairs, MAC
 * (L_A + L_B) / |com_A - com_B| < theta.                                   */
static void m_trav(sym_ctx* c, orc_node* A, orc_node* B)
{
    double dx = A->com[0] - B->com[0], dy = A->com[1] - B->com[1];
    double dist = sqrt(dx * dx + dy * dy);
    if ((A->bb_len + B->bb_len) / dist < c->theta) {
        if (A->count != 0 && B->count != 0) m_kernel_nn(c, A, B);
    } else if (A->first_child == 0) {
        for (int64_t i = A->first_part; i < (int64_t)A->first_part + A->count; i++)
            if (B->count != 0) m_trav_bhmp(c, i, B);
    } else if (B->first_child == 0) {
        for (int64_t j = B->first_part; j < (int64_t)B->first_part + B->count; j++)
            if (A->count != 0) m_trav_bhrmp(c, A, j);
    } else {
        for (uint32_t a = A->first_child; a < A->first_child + 4; a++)
            for (uint32_t b = B->first_child; b < B->first_child + 4; b++)
                if (c->nodes[a].count != 0 && c->nodes[b].count != 0) m_trav(c, &c->nodes[a], &c->nodes[b]);
    }
}

/* applyForces (:382-430): as the symmetric solver's, without the M0
 * normalisation (the kernels never applied the sink mass).                */
static void m_apply_forces(sym_ctx* c, orc_node* q)
{
    if (q->first_child != 0) {
        for (uint32_t k = q->first_child; k < q->first_child + 4; k++) {
            orc_node* ch = &c->nodes[k];
            if (ch->count == 0) continue;
            double d[2] = {ch->com[0] - q->com[0], ch->com[1] - q->com[1]};
            double e1[2], e3[4], e31[2], e2[4];
            contract2(d, q->c2, e1);
            contract3(d, q->c3, e3);
            contract2(d, e3, e31);
            for (int i = 0; i < 2; i++) ch->c1[i] += q->c1[i] + e1[i] + 0.5 * e31[i];
            for (int i = 0; i < 4; i++) e2[i] = q->c2[i] + e3[i];
            for (int i = 0; i < 4; i++) ch->c2[i] += e2[i];
            for (int i = 0; i < 8; i++) ch->c3[i] += q->c3[i];
            m_apply_forces(c, ch);
        }
    } else {
        for (int64_t p = q->first_part; p < (int64_t)q->first_part + q->count; p++) {
            double d[2] = {c->pos[2 * p] - q->com[0], c->pos[2 * p + 1] - q->com[1]};
            double e1[2], e3[4], e31[2];
            contract2(d, q->c2, e1);
            contract3(d, q->c3, e3);
            contract2(d, e3, e31);
            c->grad[2 * p] += q->c1[0] + e1[0] + 0.5 * e31[0];
            c->grad[2 * p + 1] += q->c1[1] + e1[1] + 0.5 * e31[1];
        }
    }
}

void orc_fmm_morton_solve(int kernel, double eps, double theta, const double* pos, orc_node* nodes,
                          double* grad, double* total)
{
    sym_ctx c;
    c.kernel = kernel;
    c.eps2 = eps * eps;
    c.theta = theta;
    c.pos = pos;
    c.grad = grad;
    c.nodes = nodes;
    c.total = *total;
    m_trav(&c, &nodes[0], &nodes[0]);
    m_apply_forces(&c, &nodes[0]);
    *total = c.total;
}

void orc_fmm_morton(int kernel, double eps, int max_children, int depth, double theta, int64_t n,
                    const double* pos, const double min_xy[2], const double max_xy[2],
                    uint32_t* codes_sorted, int32_t* ids_sorted, double* pos_sorted,
                    double* grad_sorted, double* total, orc_node* nodes)
{
    uint32_t d = depth >= 0 ? (uint32_t)depth : orc_get_depth(max_children, n);
    uint32_t* codes = (uint32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint32_t));
    orc_morton_codes(n, pos, min_xy, max_xy, codes);
    orc_sort_perm(n, codes, ids_sorted);
    for (int64_t k = 0; k < n; k++) {
        int32_t i = ids_sorted[k];
        codes_sorted[k] = codes[i];
        pos_sorted[2 * k] = pos[2 * i];
        pos_sorted[2 * k + 1] = pos[2 * i + 1];
    }
    free(codes);
    int64_t nn = orc_node_count(d);
    orc_node* own = NULL;
    if (!nodes) nodes = own = (orc_node*)malloc((size_t)nn * sizeof(orc_node));
    orc_build_tree(d, n, pos_sorted, min_xy, max_xy, nodes);
    if (n > 0) orc_fmm_morton_solve(kernel, eps, theta, pos_sorted, nodes, grad_sorted, total);
    free(own);
}

void orc_sym_fmm(int kernel, double eps, int max_children, int depth, double theta, int64_t n,
                 const double* pos, const double min_xy[2], const double max_xy[2],
                 uint32_t* codes_sorted, int32_t* ids_sorted, double* pos_sorted,
                 double* grad_sorted, double* total, orc_node* nodes)
{
    uint32_t d = depth >= 0 ? (uint32_t)depth : orc_get_depth(max_children, n);
    uint32_t* codes = (uint32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint32_t));
    orc_morton_codes(n, pos, min_xy, max_xy, codes);
    orc_sort_perm(n, codes, ids_sorted);
    for (int64_t k = 0; k < n; k++) {
        int32_t i = ids_sorted[k];
        codes_sorted[k] = codes[i];
        pos_sorted[2 * k] = pos[2 * i];
        pos_sorted[2 * k + 1] = pos[2 * i + 1];
    }
    free(codes);
    int64_t nn = orc_node_count(d);
    orc_node* own = NULL;
    if (!nodes) nodes = own = (orc_node*)malloc((size_t)nn * sizeof(orc_node));
    orc_build_tree(d, n, pos_sorted, min_xy, max_xy, nodes);
    if (n > 0) orc_sym_fmm_solve(kernel, eps, d, theta, n, pos_sorted, nodes, grad_sorted, total);
    free(own);
}

/* ------------------------------------------------------------------ */
/* direct sums                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    int kernel;
    double eps2;
    int64_t n;
    const double* pos;
    const int64_t* rows;
    int64_t r0, r1;
    double* grad;
    double total;
    int row_out_compact;
} naive_job;

/* TSNEnaiveKernel (nBodySolverNaive.h:124-141): uses |diff| then squares it */
static void* naive_worker(void* arg)
{
    naive_job* j = (naive_job*)arg;
    double tot = 0.0;
    for (int64_t r = j->r0; r < j->r1; r++) {
        int64_t i = j->rows ? j->rows[r] : r;
        double gx = 0.0, gy = 0.0;
        for (int64_t k = 0; k < j->n; k++) {
            if (k == i) continue;
            double dx = j->pos[2 * i] - j->pos[2 * k];
            double dy = j->pos[2 * i + 1] - j->pos[2 * k + 1];
            if (j->kernel == ORC_KERNEL_TSNE) {
                double dist = sqrt(dx * dx + dy * dy);
                double fd = 1.0 / (1.0 + (dist * dist));
                tot += fd;
                gx += fd * fd * dx;
                gy += fd * fd * dy;
            } else {
                derivs d = grav_derivs(dx * dx + dy * dy, j->eps2);
                tot += d.t;
                gx += d.D1 * dx;
                gy += d.D1 * dy;
            }
        }
        int64_t o = j->row_out_compact ? r : i;
        j->grad[2 * o] = gx;
        j->grad[2 * o + 1] = gy;
    }
    j->total = tot;
    return NULL;
}

static void run_rows(int kernel, double eps, int64_t n, const double* pos, int64_t m,
                     const int64_t* rows, double* grad, double* total, int nthreads, int compact)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    naive_job jobs[256];
    int64_t chunk = (m + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        jobs[t].kernel = kernel;
        jobs[t].eps2 = eps * eps;
        jobs[t].n = n;
        jobs[t].pos = pos;
        jobs[t].rows = rows;
        jobs[t].r0 = t * chunk < m ? t * chunk : m;
        jobs[t].r1 = (t + 1) * chunk < m ? (t + 1) * chunk : m;
        jobs[t].grad = grad;
        jobs[t].total = 0.0;
        jobs[t].row_out_compact = compact;
        pthread_create(&th[t], NULL, naive_worker, &jobs[t]);
    }
    double tot = 0.0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        tot += jobs[t].total;
    }
    if (total) *total = tot;
}

void orc_naive(int kernel, double eps, int64_t n, const double* pos, double* grad,
               double* total, int nthreads)
{
    run_rows(kernel, eps, n, pos, n, NULL, grad, total, nthreads, 0);
}

void orc_direct_rows(int kernel, double eps, int64_t n, const double* pos, int64_t m,
                     const int64_t* idx, double* grad_rows, int nthreads)
{
    run_rows(kernel, eps, n, pos, m, idx, grad_rows, NULL, nthreads, 1);
}

/* ------------------------------------------------------------------ */
/* Barnes-Hut (pointer quadtree)                                       */
/* ------------------------------------------------------------------ */

typedef struct bh_node {
    float total_mass;        /* QuadTree::totalMass is float (quadtree.h:17) */
    double com[2];
    double lo[2], hi[2];
    int32_t* occ;
    int64_t nocc;
    struct bh_node* ch[4];
    int nch;
} bh_node;

/* QuadTree::createTree (quadtree.h:100-172).  The return value is
 * std::pair<float, glm::vec2>, so the parent sees float-rounded child COMs. */
static void bh_create(bh_node* q, const double* pos, int maxc, float* ret_m, float ret_c[2])
{
    if (q->nocc > maxc) {
        int32_t* part[4];
        int64_t cnt[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++) part[k] = (int32_t*)malloc((size_t)q->nocc * sizeof(int32_t));
        double l = (q->hi[0] - q->lo[0]) / 2.0;
        double mx = q->lo[0] + l, my = q->lo[1] + l;
        for (int64_t i = 0; i < q->nocc; i++) {
            int32_t id = q->occ[i];
            double x = pos[2 * id], y = pos[2 * id + 1];
            int k;
            if (x >= mx && y >= my) k = 0;          /* HH */
            else if (x >= mx && y < my) k = 1;      /* HL */
            else if (x < mx && y >= my) k = 2;      /* LH */
            else k = 3;                             /* LL */
            part[k][cnt[k]++] = id;
        }
        double blo[4][2] = {{mx, my}, {mx, q->lo[1]}, {q->lo[0], my}, {q->lo[0], q->lo[1]}};
        double bhi[4][2] = {{q->hi[0], q->hi[1]}, {q->hi[0], my}, {mx, q->hi[1]}, {mx, my}};
        q->nch = 0;
        for (int k = 0; k < 4; k++) {
            if (cnt[k] == 0) {
                free(part[k]);
                continue;
            }
            bh_node* c = (bh_node*)calloc(1, sizeof(bh_node));
            c->occ = part[k];
            c->nocc = cnt[k];
            c->lo[0] = blo[k][0]; c->lo[1] = blo[k][1];
            c->hi[0] = bhi[k][0]; c->hi[1] = bhi[k][1];
            q->ch[q->nch++] = c;
        }
        q->total_mass = 0.0f;
        q->com[0] = q->com[1] = 0.0;
        for (int k = 0; k < q->nch; k++) {
            float cm, cc[2];
            bh_create(q->ch[k], pos, maxc, &cm, cc);
            double m = (double)cm;
            q->total_mass = (float)((double)q->total_mass + m);
            q->com[0] += m * (double)cc[0];
            q->com[1] += m * (double)cc[1];
        }
    } else {
        q->total_mass = 0.0f;
        q->com[0] = q->com[1] = 0.0;
        for (int64_t i = 0; i < q->nocc; i++) {
            q->total_mass = (float)((double)q->total_mass + 1.0);
            q->com[0] += 1.0 * pos[2 * q->occ[i]];
            q->com[1] += 1.0 * pos[2 * q->occ[i] + 1];
        }
    }
    q->com[0] /= (double)q->total_mass;
    q->com[1] /= (double)q->total_mass;
    *ret_m = q->total_mass;
    ret_c[0] = (float)q->com[0];
    ret_c[1] = (float)q->com[1];
}

static void bh_free(bh_node* q)
{
    for (int k = 0; k < q->nch; k++) {
        bh_free(q->ch[k]);
        free(q->ch[k]);
    }
    free(q->occ);
}

typedef struct {
    int kernel;
    double eps2;
    double theta;
    const double* pos;
    double total;
} bh_ctx;

/* NBodySolverBH::traverseBH (nBodySolverBH.h:56-89) + TSNEBHPNKernel /
 * TSNEBHPPKernel (:94-116); gravity uses the softened kernel.             */
static void bh_trav(bh_ctx* c, int64_t p, const bh_node* q, double* g)
{
    double l = q->hi[0] - q->lo[0];
    double dx = c->pos[2 * p] - q->com[0], dy = c->pos[2 * p + 1] - q->com[1];
    double len = sqrt(dx * dx + dy * dy);
    if (l / len < c->theta) {
        double sq = dx * dx + dy * dy;
        double tm = (double)q->total_mass;
        if (c->kernel == ORC_KERNEL_TSNE) {
            double fd = 1.0 / (1.0 + sq);
            c->total += tm * fd;
            g[0] += tm * fd * fd * dx;
            g[1] += tm * fd * fd * dy;
        } else {
            derivs d = grav_derivs(sq, c->eps2);
            c->total += tm * d.t;
            g[0] += tm * d.D1 * dx;
            g[1] += tm * d.D1 * dy;
        }
    } else if (q->nch <= 1) {
        for (int64_t i = 0; i < q->nocc; i++) {
            int64_t o = q->occ[i];
            if (o == p) continue;
            double ex = c->pos[2 * p] - c->pos[2 * o], ey = c->pos[2 * p + 1] - c->pos[2 * o + 1];
            double sq = ex * ex + ey * ey;
            if (c->kernel == ORC_KERNEL_TSNE) {
                double fd = 1.0 / (1.0 + sq);
                c->total += fd;
                g[0] += fd * fd * ex;
                g[1] += fd * fd * ey;
            } else {
                derivs d = grav_derivs(sq, c->eps2);
                c->total += d.t;
                g[0] += d.D1 * ex;
                g[1] += d.D1 * ey;
            }
        }
    } else {
        for (int k = 0; k < q->nch; k++) bh_trav(c, p, q->ch[k], g);
    }
}

int orc_bh(int kernel, double eps, int max_children, double theta, int64_t n,
           const double* pos, double* grad, double* total)
{
    if (n <= 0) {
        if (total) *total = 0.0;
        return 0;
    }
    bh_node root;
    memset(&root, 0, sizeof(root));
    root.occ = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    root.nocc = n;
    double lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; i++) {
        root.occ[i] = (int32_t)i;
        for (int a = 0; a < 2; a++) {
            lo[a] = dmin(lo[a], pos[2 * i + a]);
            hi[a] = dmax(hi[a], pos[2 * i + a]);
        }
    }
    double ld = dmax(hi[0] - lo[0], hi[1] - lo[1]);
    root.lo[0] = lo[0];
    root.lo[1] = lo[1];
    root.hi[0] = lo[0] + ld + 0.0001;
    root.hi[1] = lo[1] + ld + 0.0001;
    float m, cc[2];
    bh_create(&root, pos, max_children, &m, cc);
    bh_ctx c = {kernel, eps * eps, theta, pos, 0.0};
    for (int64_t i = 0; i < n; i++) {
        grad[2 * i] = grad[2 * i + 1] = 0.0;
        bh_trav(&c, i, &root, grad + 2 * i);
    }
    if (total) *total = c.total;
    bh_free(&root);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Barnes-Hut with quadrupoles: NBodySolverBHMP + QuadTreeMultiPole    */
/* ------------------------------------------------------------------ */

typedef struct bhmp_node {
    double mass;             /* QuadTreeMultiPole::totalMass (double)          */
    double com[2];
    double quad[4];          /* quadrupole (row-major 2x2)                     */
    double lo[2], hi[2];
    int32_t* occ;
    int64_t nocc;
    struct bhmp_node* ch[4];
    int nch;
} bhmp_node;

/* QuadTreeMultiPole::createTree (quadtreemultipole.h:174-289): the same split
 * as QuadTree, FP64 masses and COMs, quadrupole sum_c [M_c (dc dc^T) + Q_c]. */
static void bhmp_create(bhmp_node* q, const double* pos, int maxc)
{
    if (q->nocc > maxc) {
        int32_t* part[4];
        int64_t cnt[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++) part[k] = (int32_t*)malloc((size_t)q->nocc * sizeof(int32_t));
        double l = (q->hi[0] - q->lo[0]) / 2.0;
        double mx = q->lo[0] + l, my = q->lo[1] + l;
        for (int64_t i = 0; i < q->nocc; i++) {
            int32_t id = q->occ[i];
            double x = pos[2 * id], y = pos[2 * id + 1];
            int k;
            if (x >= mx && y >= my) k = 0;          /* HH */
            else if (x >= mx && y < my) k = 1;      /* HL */
            else if (x < mx && y >= my) k = 2;      /* LH */
            else k = 3;                             /* LL */
            part[k][cnt[k]++] = id;
        }
        double blo[4][2] = {{mx, my}, {mx, q->lo[1]}, {q->lo[0], my}, {q->lo[0], q->lo[1]}};
        double bhi[4][2] = {{q->hi[0], q->hi[1]}, {q->hi[0], my}, {mx, q->hi[1]}, {mx, my}};
        q->nch = 0;
        for (int k = 0; k < 4; k++) {
            if (cnt[k] == 0) {
                free(part[k]);
                continue;
            }
            bhmp_node* c = (bhmp_node*)calloc(1, sizeof(bhmp_node));
            c->occ = part[k];
            c->nocc = cnt[k];
            c->lo[0] = blo[k][0]; c->lo[1] = blo[k][1];
            c->hi[0] = bhi[k][0]; c->hi[1] = bhi[k][1];
            q->ch[q->nch++] = c;
        }
        q->mass = 0.0;
        q->com[0] = q->com[1] = 0.0;
        for (int k = 0; k < q->nch; k++) {
            bhmp_create(q->ch[k], pos, maxc);
            q->mass += q->ch[k]->mass;
            q->com[0] += q->ch[k]->mass * q->ch[k]->com[0];
            q->com[1] += q->ch[k]->mass * q->ch[k]->com[1];
        }
        q->com[0] /= q->mass;
        q->com[1] /= q->mass;
        for (int i = 0; i < 4; i++) q->quad[i] = 0.0;
        for (int k = 0; k < q->nch; k++) {
            const bhmp_node* c = q->ch[k];
            double rx = c->com[0] - q->com[0], ry = c->com[1] - q->com[1];
            double o[4] = {rx * rx, rx * ry, ry * rx, ry * ry};
            for (int i = 0; i < 4; i++) q->quad[i] += c->mass * o[i];
            for (int i = 0; i < 4; i++) q->quad[i] += c->quad[i];
        }
    } else {
        q->mass = 0.0;
        q->com[0] = q->com[1] = 0.0;
        for (int64_t i = 0; i < q->nocc; i++) {
            q->mass += 1.0;
            q->com[0] += 1.0 * pos[2 * q->occ[i]];
            q->com[1] += 1.0 * pos[2 * q->occ[i] + 1];
        }
        q->com[0] /= q->mass;
        q->com[1] /= q->mass;
        for (int i = 0; i < 4; i++) q->quad[i] = 0.0;
        for (int64_t i = 0; i < q->nocc; i++) {
            double rx = pos[2 * q->occ[i]] - q->com[0], ry = pos[2 * q->occ[i] + 1] - q->com[1];
            double o[4] = {rx * rx, rx * ry, ry * rx, ry * ry};
            for (int j = 0; j < 4; j++) q->quad[j] += o[j];
        }
    }
}

static void bhmp_free(bhmp_node* q)
{
    for (int k = 0; k < q->nch; k++) {
        bhmp_free(q->ch[k]);
        free(q->ch[k]);
    }
    free(q->occ);
}

/* NBodySolverBHMP::traverseBHMP (nBodySolverBHMP.h:59-93) + TSNEBHMPPNKernel
 * / TSNEBHMPPPKernel (:97-135); gravity puts the softened kernel in the same
 * slots (C1 with the source quadrupole).                                   */
static void bhmp_trav(bh_ctx* c, int64_t p, const bhmp_node* q, double* g)
{
    double l = q->hi[0] - q->lo[0];
    double dx = c->pos[2 * p] - q->com[0], dy = c->pos[2 * p + 1] - q->com[1];
    double len = sqrt(dx * dx + dy * dy);
    if (l / len < c->theta) {
        double sq = dx * dx + dy * dy;
        double C1[2];
        derivs d;
        if (c->kernel == ORC_KERNEL_TSNE) {
            double rS = 1.0 + sq;
            d.D1 = 1.0 / (rS * rS);
            d.D2 = -4.0 / (rS * rS * rS);
            d.D3 = 24.0 / (rS * rS * rS * rS);
            c->total += q->mass / rS;
        } else {
            d = grav_derivs(sq, c->eps2);
            c->total += q->mass * d.t;
        }
        far_c1(dx, dy, q->mass, q->quad, d.D1, d.D2, d.D3, C1);
        g[0] += C1[0];
        g[1] += C1[1];
    } else if (q->nch <= 1) {
        for (int64_t i = 0; i < q->nocc; i++) {
            int64_t o = q->occ[i];
            if (o == p) continue;
            double ex = c->pos[2 * p] - c->pos[2 * o], ey = c->pos[2 * p + 1] - c->pos[2 * o + 1];
            double sq = ex * ex + ey * ey;
            if (c->kernel == ORC_KERNEL_TSNE) {
                double fd = 1.0 / (1.0 + sq);
                c->total += fd;
                g[0] += fd * fd * ex;
                g[1] += fd * fd * ey;
            } else {
                derivs d = grav_derivs(sq, c->eps2);
                c->total += d.t;
                g[0] += d.D1 * ex;
                g[1] += d.D1 * ey;
            }
        }
    } else {
        for (int k = 0; k < q->nch; k++) bhmp_trav(c, p, q->ch[k], g);
    }
}

int orc_bhmp(int kernel, double eps, int max_children, double theta, int64_t n,
             const double* pos, double* grad, double* total)
{
    if (n <= 0) {
        if (total) *total = 0.0;
        return 0;
    }
    bhmp_node root;
    memset(&root, 0, sizeof(root));
    root.occ = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    root.nocc = n;
    double lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; i++) {
        root.occ[i] = (int32_t)i;
        for (int a = 0; a < 2; a++) {
            lo[a] = dmin(lo[a], pos[2 * i + a]);
            hi[a] = dmax(hi[a], pos[2 * i + a]);
        }
    }
    double ld = dmax(hi[0] - lo[0], hi[1] - lo[1]);
    root.lo[0] = lo[0];
    root.lo[1] = lo[1];
    root.hi[0] = lo[0] + ld + 0.0001;
    root.hi[1] = lo[1] + ld + 0.0001;
    bhmp_create(&root, pos, max_children);
    bh_ctx c = {kernel, eps * eps, theta, pos, 0.0};
    for (int64_t i = 0; i < n; i++) {
        grad[2 * i] = grad[2 * i + 1] = 0.0;
        bhmp_trav(&c, i, &root, grad + 2 * i);
    }
    if (total) *total = c.total;
    bhmp_free(&root);
    return 0;
}

/* ------------------------------------------------------------------ */
/* t-SNE composition                                                   */
/* ------------------------------------------------------------------ */

void orc_tsne_attractive(int64_t n, const uint32_t* row_ptr, const uint32_t* col,
                         const double* val, const double* pos, double exag, double* grad)
{
    for (int64_t r = 0; r < n; r++) {
        double ax = 0.0, ay = 0.0;
        for (uint32_t i = row_ptr[r]; i < row_ptr[r + 1]; i++) {
            uint32_t c = col[i];
            double dx = pos[2 * c] - pos[2 * r];
            double dy = pos[2 * c + 1] - pos[2 * r + 1];
            double d = dx * dx + dy * dy;
            double q = 1.0 / (1.0 + d);
            ax += exag * val[i] * q * dx;
            ay += exag * val[i] * q * dy;
        }
        grad[2 * r] += ax;
        grad[2 * r + 1] += ay;
    }
}

void orc_tsne_step(int64_t n, const double* y, const double* y_prev, const uint32_t* row_ptr,
                   const uint32_t* col, const double* val, int max_children, int depth,
                   double theta, double exag_code, double lr, double momentum, double* y_next,
                   double* grad_out, double* z_out)
{
    double mn[2] = {INFINITY, INFINITY}, mx[2] = {-INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; i++)
        for (int a = 0; a < 2; a++) {
            mn[a] = dmin(mn[a], y[2 * i + a]);
            mx[a] = dmax(mx[a], y[2 * i + a]);
        }
    uint32_t* cs = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    int32_t* ids = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    double* ps = (double*)malloc((size_t)n * 2 * sizeof(double));
    double* gs = (double*)calloc((size_t)n * 2, sizeof(double));
    double z = 0.0;
    orc_sym_fmm(ORC_KERNEL_TSNE, 0.0, max_children, depth, theta, n, y, mn, mx, cs, ids, ps, gs, &z, NULL);
    double s = 4.0 / z; /* updateRepulsive (tsne.h:287-301) */
    for (int64_t k = 0; k < n; k++) {
        grad_out[2 * ids[k]] = gs[2 * k] * s;
        grad_out[2 * ids[k] + 1] = gs[2 * k + 1] * s;
    }
    orc_tsne_attractive(n, row_ptr, col, val, y, exag_code, grad_out);
    for (int64_t i = 0; i < 2 * n; i++) /* updatePoints (tsne.h:179-206) */
        y_next[i] = y[i] + lr * grad_out[i] + momentum * (y[i] - y_prev[i]);
    if (z_out) *z_out = z;
    free(cs);
    free(ids);
    free(ps);
    free(gs);
}

/* ------------------------------------------------------------------ particle mesh
 * NBodySolverPM::computeFftGradient (nBodySolverPM.h:763-1039) with its helpers
 * precompute_2d (:686-760), n_body_fft_2d (:413-682) and interpolate (:380-410):
 * the published FFT-accelerated interpolation scheme (Linderman et al.,
 * FIt-SNE).  The square [min, max]^2 holds nb x nb boxes of p Lagrange nodes per
 * dimension (p equispaced nodes at (k + 1/2)/p of the box); the charges
 * (1, x, y, x^2 + y^2) are spread to the nodes, convolved with the squared
 * Cauchy kernel (1 + r^2)^-2 on the uniform node grid through a zero-padded 2D
 * DFT (a plain row/column DFT here; FFTW in the reference), and interpolated
 * back.  min/max follow the reference's single pass with `else if`: a value
 * that raises the running maximum is never taken for the minimum.           */
typedef struct {
    double re, im;
} orc_c;

static void pm_dft_r2c(int n, const double* in, orc_c* out, const double* cs, const double* sn)
{
    /* n x n real -> n x (n/2+1) complex, exp(-2 pi i (ia + kb)/n) */
    const int h = n / 2 + 1;
    orc_c* rows = (orc_c*)malloc((size_t)n * h * sizeof(orc_c));
    for (int a = 0; a < n; a++)
        for (int k = 0; k < h; k++) {
            double re = 0.0, im = 0.0;
            for (int b = 0; b < n; b++) {
                const int t = (int)(((int64_t)k * b) % n);
                re += in[(size_t)a * n + b] * cs[t];
                im -= in[(size_t)a * n + b] * sn[t];
            }
            rows[(size_t)a * h + k].re = re;
            rows[(size_t)a * h + k].im = im;
        }
    for (int k = 0; k < h; k++)
        for (int i = 0; i < n; i++) {
            double re = 0.0, im = 0.0;
            for (int a = 0; a < n; a++) {
                const int t = (int)(((int64_t)i * a) % n);
                const orc_c v = rows[(size_t)a * h + k];
                re += v.re * cs[t] + v.im * sn[t];
                im += v.im * cs[t] - v.re * sn[t];
            }
            out[(size_t)i * h + k].re = re;
            out[(size_t)i * h + k].im = im;
        }
    free(rows);
}

static void pm_dft_c2r(int n, const orc_c* in, double* out, const double* cs, const double* sn)
{
    /* unnormalised inverse of pm_dft_r2c */
    const int h = n / 2 + 1;
    orc_c* cols = (orc_c*)malloc((size_t)n * h * sizeof(orc_c));
    for (int k = 0; k < h; k++)
        for (int a = 0; a < n; a++) {
            double re = 0.0, im = 0.0;
            for (int i = 0; i < n; i++) {
                const int t = (int)(((int64_t)i * a) % n);
                const orc_c v = in[(size_t)i * h + k];
                re += v.re * cs[t] - v.im * sn[t];
                im += v.im * cs[t] + v.re * sn[t];
            }
            cols[(size_t)a * h + k].re = re;
            cols[(size_t)a * h + k].im = im;
        }
    for (int a = 0; a < n; a++)
        for (int b = 0; b < n; b++) {
            double s = cols[(size_t)a * h].re;
            int kmax = h - 1;
            if (n % 2 == 0) {
                s += cols[(size_t)a * h + n / 2].re * ((b & 1) ? -1.0 : 1.0);
                kmax = n / 2 - 1;
            }
            for (int k = 1; k <= kmax; k++) {
                const int t = (int)(((int64_t)k * b) % n);
                const orc_c v = cols[(size_t)a * h + k];
                s += 2.0 * (v.re * cs[t] - v.im * sn[t]);
            }
            out[(size_t)a * n + b] = s;
        }
    free(cols);
}

/* Lagrange basis values of the p nodes sp[] at t (interpolate, :380-410) */
static void pm_lagrange(int p, const double* sp, const double* den, double t, double* v)
{
    for (int j = 0; j < p; j++) {
        double num = 1.0;
        for (int k = 0; k < p; k++)
            if (j != k) num *= t - sp[k];
        v[j] = num / den[j];
    }
}

int orc_pm(int p, double cell_size, int min_intervals, int64_t n, const double* pos, double* grad,
           double* total)
{
    if (n <= 0 || p < 1 || p > 16) return -1;
    const double inf = (double)(float)(1e300 * 1e300);
    double mn = inf, mx = -inf;
    for (int64_t i = 0; i < n; i++)
        for (int a = 0; a < 2; a++) {
            const double v = pos[2 * i + a];
            if (v > mx) mx = v;
            else if (v < mn) mn = v;
        }
    int nb = (int)((mx - mn) / cell_size);
    if (nb < min_intervals) nb = min_intervals;
    const double bw = (mx - mn) / (double)nb;
    /* node spacings inside a box, and the node coordinates of the whole grid */
    double sp[16], den[16];
    const double hs = 1.0 / (double)p;
    sp[0] = hs / 2;
    for (int i = 1; i < p; i++) sp[i] = sp[i - 1] + hs;
    for (int i = 0; i < p; i++) {
        den[i] = 1.0;
        for (int j = 0; j < p; j++)
            if (i != j) den[i] *= sp[i] - sp[j];
    }
    const int n1 = p * nb, nf = 2 * n1, hf = nf / 2 + 1;
    double* xt = (double*)malloc((size_t)n1 * sizeof(double));
    const double hw = hs * bw;
    xt[0] = mn + hw / 2;
    for (int i = 1; i < n1; i++) xt[i] = xt[i - 1] + hw;
    /* the kernel on the node grid, mirrored into the zero-padded circulant generator */
    double* cs = (double*)malloc((size_t)nf * sizeof(double));
    double* sn = (double*)malloc((size_t)nf * sizeof(double));
    for (int t = 0; t < nf; t++) {
        const double ang = 2.0 * 3.14159265358979323846 * (double)t / (double)nf;
        cs[t] = cos(ang);
        sn[t] = sin(ang);
    }
    double* kt = (double*)calloc((size_t)nf * nf, sizeof(double));
    for (int i = 0; i < n1; i++)
        for (int j = 0; j < n1; j++) {
            const double dy = xt[0] - xt[i], dx = xt[0] - xt[j];
            const double v = pow(1.0 + pow(dy, 2) + pow(dx, 2), -2);
            kt[(size_t)(n1 + i) * nf + (n1 + j)] = v;
            kt[(size_t)(n1 - i) * nf + (n1 + j)] = v;
            kt[(size_t)(n1 + i) * nf + (n1 - j)] = v;
            kt[(size_t)(n1 - i) * nf + (n1 - j)] = v;
        }
    orc_c* kf = (orc_c*)malloc((size_t)nf * hf * sizeof(orc_c));
    pm_dft_r2c(nf, kt, kf, cs, sn);
    /* boxes, in-box coordinates and interpolation weights of every point */
    int* bx = (int*)malloc((size_t)n * sizeof(int));
    int* by = (int*)malloc((size_t)n * sizeof(int));
    double* wx = (double*)malloc((size_t)n * p * sizeof(double));
    double* wy = (double*)malloc((size_t)n * p * sizeof(double));
    for (int64_t i = 0; i < n; i++) {
        const double x = pos[2 * i], y = pos[2 * i + 1];
        int ix = (int)((x - mn) / bw), iy = (int)((y - mn) / bw);
        ix = ix >= nb ? nb - 1 : (ix < 0 ? 0 : ix);
        iy = iy >= nb ? nb - 1 : (iy < 0 ? 0 : iy);
        bx[i] = ix;
        by[i] = iy;
        const double x0 = ix * bw + mn, y0 = iy * bw + mn;
        pm_lagrange(p, sp, den, (x - x0) / bw, wx + (size_t)i * p);
        pm_lagrange(p, sp, den, (y - y0) / bw, wy + (size_t)i * p);
    }
    /* spread the four charges: node row = x node, column = y node */
    double* w = (double*)calloc((size_t)n1 * n1 * 4, sizeof(double));
    for (int64_t i = 0; i < n; i++) {
        const double x = pos[2 * i], y = pos[2 * i + 1];
        const double q[4] = {1.0, x, y, x * x + y * y};
        for (int a = 0; a < p; a++)
            for (int b = 0; b < p; b++) {
                const size_t idx = (size_t)(bx[i] * p + a) * n1 + (size_t)(by[i] * p + b);
                for (int d = 0; d < 4; d++) w[idx * 4 + d] += wy[(size_t)i * p + b] * wx[(size_t)i * p + a] * q[d];
            }
    }
    /* convolve each charge with the kernel */
    double* fin = (double*)malloc((size_t)nf * nf * sizeof(double));
    orc_c* fw = (orc_c*)malloc((size_t)nf * hf * sizeof(orc_c));
    double* fout = (double*)malloc((size_t)nf * nf * sizeof(double));
    double* pot_grid = (double*)malloc((size_t)n1 * n1 * 4 * sizeof(double));
    for (int d = 0; d < 4; d++) {
        memset(fin, 0, (size_t)nf * nf * sizeof(double));
        for (int i = 0; i < n1; i++)
            for (int j = 0; j < n1; j++) fin[(size_t)i * nf + j] = w[((size_t)i * n1 + j) * 4 + d];
        pm_dft_r2c(nf, fin, fw, cs, sn);
        for (size_t k = 0; k < (size_t)nf * hf; k++) {
            const double x_ = fw[k].re, y_ = fw[k].im, u_ = kf[k].re, v_ = kf[k].im;
            fw[k].re = x_ * u_ - y_ * v_;
            fw[k].im = x_ * v_ + y_ * u_;
        }
        pm_dft_c2r(nf, fw, fout, cs, sn);
        for (int i = 0; i < n1; i++)
            for (int j = 0; j < n1; j++)
                pot_grid[((size_t)i * n1 + j) * 4 + d] = fout[(size_t)(n1 + i) * nf + (n1 + j)] / (double)((int64_t)nf * nf);
    }
    /* interpolate the potentials back, then Z and the repulsive gradient */
    double sum_q = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double phi[4] = {0.0, 0.0, 0.0, 0.0};
        for (int a = 0; a < p; a++)
            for (int b = 0; b < p; b++) {
                const size_t idx = (size_t)(bx[i] * p + a) * n1 + (size_t)(by[i] * p + b);
                for (int d = 0; d < 4; d++)
                    phi[d] += wx[(size_t)i * p + a] * wy[(size_t)i * p + b] * pot_grid[idx * 4 + d];
            }
        const double x = pos[2 * i], y = pos[2 * i + 1];
        sum_q += (1 + x * x + y * y) * phi[0] - 2 * (x * phi[1] + y * phi[2]) + phi[3];
        /* the reference stores dC = -(x phi1 - phi2) and returns derivative = -dC */
        grad[2 * i] = x * phi[0] - phi[1];
        grad[2 * i + 1] = y * phi[0] - phi[2];
    }
    *total = sum_q - (double)n;
    free(xt);
    free(cs);
    free(sn);
    free(kt);
    free(kf);
    free(bx);
    free(by);
    free(wx);
    free(wy);
    free(w);
    free(fin);
    free(fw);
    free(fout);
    free(pot_grid);
    return 0;
}

/* ------------------------------------------------------------------ affinities
 * The t-SNE affinity matrix the reference reads from openTSNE's output
 * (MnistLoader.ipynb cell 14: PerplexityBasedNN, k = 3 * perplexity,
 * symmetrize=True; CSR by TSNE::setupEfficientPmatrix, tsne.h:462-520).
 * openTSNE is absent, so the published algorithm is restated with every
 * operation fixed (fused only where fma/fmaf is written; this file is built
 * with -ffp-contract=off): FP32 squared distances summed over the dimensions
 * in order, neighbours ordered by (distance, index); per-row FP64 bisection
 * of the bandwidth to the perplexity with exp and log written from their
 * series; (P + P^T) / (2N) with the two contributions to an entry added.   */

static const double A_LN2_HI = 0x1.62e42fee00000p-1;
static const double A_LN2_LO = 0x1.a39ef35793c76p-33;
static const double A_INV_LN2 = 0x1.71547652b82fep+0;

static double a_scale2(double v, int k)
{
    uint64_t b;
    double f;
    if (k < -1000) {
        v *= 0x1p-600;
        k += 600;
    }
    b = (uint64_t)(k + 1023) << 52;
    memcpy(&f, &b, 8);
    return v * f;
}

double orc_exp(double x)
{
    double kf, r, q;
    int k;
    if (!(x > -745.0)) return 0.0;
    if (x > 709.0) return INFINITY;
    kf = floor(x * A_INV_LN2 + 0.5);
    k = (int)kf;
    r = fma(-kf, A_LN2_HI, x);
    r = fma(-kf, A_LN2_LO, r);
    /* Taylor series of e^r to degree 13 (|r| <= ln 2 / 2), Horner form */
    q = 0x1.6124613a86d09p-33;
    q = fma(q, r, 0x1.1eed8eff8d898p-29);
    q = fma(q, r, 0x1.ae64567f544e4p-26);
    q = fma(q, r, 0x1.27e4fb7789f5cp-22);
    q = fma(q, r, 0x1.71de3a556c734p-19);
    q = fma(q, r, 0x1.a01a01a01a01ap-16);
    q = fma(q, r, 0x1.a01a01a01a01ap-13);
    q = fma(q, r, 0x1.6c16c16c16c17p-10);
    q = fma(q, r, 0x1.1111111111111p-7);
    q = fma(q, r, 0x1.5555555555555p-5);
    q = fma(q, r, 0x1.5555555555555p-3);
    q = fma(q, r, 0.5);
    q = fma(q, r, 1.0);
    q = fma(q, r, 1.0);
    return a_scale2(q, k);
}

double orc_log(double x)
{
    uint64_t b;
    double m, z, z2, q, lm, ed;
    int e;
    memcpy(&b, &x, 8);
    e = (int)((b >> 52) & 0x7FF) - 1023;
    b = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
    memcpy(&m, &b, 8);
    if (m > 1.4142135623730951) {
        m *= 0.5;
        e += 1;
    }
    /* log m = 2 atanh((m - 1)/(m + 1)), odd series to z^27 */
    z = (m - 1.0) / (m + 1.0);
    z2 = z * z;
    q = 0.037037037037037035;
    q = fma(q, z2, 0.04);
    q = fma(q, z2, 0.043478260869565216);
    q = fma(q, z2, 0.047619047619047616);
    q = fma(q, z2, 0.05263157894736842);
    q = fma(q, z2, 0.058823529411764705);
    q = fma(q, z2, 0.06666666666666667);
    q = fma(q, z2, 0.07692307692307693);
    q = fma(q, z2, 0.09090909090909091);
    q = fma(q, z2, 0.1111111111111111);
    q = fma(q, z2, 0.14285714285714285);
    q = fma(q, z2, 0.2);
    q = fma(q, z2, 0.3333333333333333);
    lm = 2.0 * fma(z * z2, q, z);
    ed = (double)e;
    return fma(ed, A_LN2_HI, fma(ed, A_LN2_LO, lm));
}

static int a_before(float da, int32_t ja, float db, int32_t jb)
{
    return da < db || (da == db && ja < jb);
}

void orc_knn(int64_t n, int dim, const float* x, int k, float* dist, int32_t* idx)
{
    for (int64_t i = 0; i < n; i++) {
        float* rd = dist + i * k;
        int32_t* ri = idx + i * k;
        int cnt = 0;
        for (int64_t j = 0; j < n; j++) {
            float d = 0.f;
            int pos, e;
            if (j == i) continue;
            for (int t = 0; t < dim; t++) {
                const float df = x[i * dim + t] - x[j * dim + t];
                d = fmaf(df, df, d);
            }
            if (cnt == k && !a_before(d, (int32_t)j, rd[k - 1], ri[k - 1])) continue;
            pos = 0;
            while (pos < cnt && a_before(rd[pos], ri[pos], d, (int32_t)j)) pos++;
            e = cnt < k ? cnt : k - 1;
            for (; e > pos; e--) {
                rd[e] = rd[e - 1];
                ri[e] = ri[e - 1];
            }
            rd[pos] = d;
            ri[pos] = (int32_t)j;
            if (cnt < k) cnt++;
        }
    }
}

void orc_perplexity(int64_t n, int k, const float* dist, double perplexity, int max_iter, double tol, double* p)
{
    const double log_perp = orc_log(perplexity);
    for (int64_t i = 0; i < n; i++) {
        const float* d = dist + i * k;
        const double dmin = (double)d[0];
        double beta = 1.0, lo = 0.0, hi = INFINITY, s;
        for (int it = 0; it < max_iter; it++) {
            double ss = 0.0, sd = 0.0, h, diff;
            for (int j = 0; j < k; j++) {
                const double dj = (double)d[j] - dmin;
                const double w = orc_exp(-dj * beta);
                ss += w;
                sd = fma(dj, w, sd);
            }
            h = orc_log(ss) + beta * sd / ss;
            diff = h - log_perp;
            if (fabs(diff) < tol) break;
            if (diff > 0.0) {
                lo = beta;
                beta = isinf(hi) ? beta * 2.0 : (lo + hi) * 0.5;
            } else {
                hi = beta;
                beta = (lo + hi) * 0.5;
            }
        }
        s = 0.0;
        for (int j = 0; j < k; j++) s += orc_exp(-((double)d[j] - dmin) * beta);
        for (int j = 0; j < k; j++) p[i * k + j] = orc_exp(-((double)d[j] - dmin) * beta) / s;
    }
}

typedef struct {
    uint32_t row, col;
    int64_t e;
    double v;
} a_entry;

static int a_cmp(const void* a, const void* b)
{
    const a_entry* x = (const a_entry*)a;
    const a_entry* y = (const a_entry*)b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return x->e < y->e ? -1 : (x->e > y->e);
}

int64_t orc_symmetrize(int64_t n, int k, const int32_t* idx, const double* p, uint32_t* row_ptr, uint32_t* col,
                       double* val)
{
    const int64_t nk = n * k, m = 2 * nk;
    const double c = 1.0 / (2.0 * (double)n);
    a_entry* t = (a_entry*)malloc((size_t)m * sizeof(a_entry));
    int64_t u = 0;
    for (int64_t e = 0; e < nk; e++) {
        const double w = p[e] * c;
        t[e].row = (uint32_t)(e / k);
        t[e].col = (uint32_t)idx[e];
        t[e].e = e;
        t[e].v = w;
        t[nk + e].row = (uint32_t)idx[e];
        t[nk + e].col = (uint32_t)(e / k);
        t[nk + e].e = nk + e;
        t[nk + e].v = w;
    }
    qsort(t, (size_t)m, sizeof(a_entry), a_cmp);
    for (int64_t q = 0; q < m; q++) {
        if (q > 0 && t[q].row == t[q - 1].row && t[q].col == t[q - 1].col) {
            val[u - 1] = val[u - 1] + t[q].v;
            continue;
        }
        if (q == 0 || t[q].row != t[q - 1].row) row_ptr[t[q].row] = (uint32_t)u;
        col[u] = t[q].col;
        val[u] = t[q].v;
        u++;
    }
    row_ptr[n] = (uint32_t)u;
    free(t);
    return u;
}
