/*
 * ORACLE — test infrastructure, not the product.  See amr_oracle.h.
 *
 * Plain-C restatement of the gpu-amr reference (paths within the reference
 * project).  Data layout follows the reference exactly: per leaf one padded
 * patch of (n+2h)^rank doubles, row-major, layout dim 0 slowest, physical x
 * on the last (fastest) layout index (physics_system.hpp:33-42).
 */
#include "amr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { NB_NONE = 0, NB_SAME = 1, NB_FINER = 2, NB_COARSER = 3 };
enum { ST_STABLE = 0, ST_REFINE = 1, ST_COARSEN = 2 };

/* ------------------------------------------------------------------ hash */
/* SplitMix64 finaliser (public algorithm by S. Vigna). */
static uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

double oracle_unit_hash(uint64_t a, uint64_t b, uint64_t c)
{
    const uint64_t h = mix64(a ^ mix64(b ^ mix64(c)));
    return (double)(h >> 11) * 0x1.0p-53;
}

/* ---------------------------------------------------------------- morton */
/* Bit interleave from its definition: coordinate k of a rank-r point sits at
 * bit positions r*b + k (x lowest), as libmorton's 64-bit encoders lay it out
 * (lib/libmorton/morton2D.h, morton3D.h).  Spreads by binary magic numbers. */
static uint64_t spread2(uint64_t v) /* one zero between bits */
{
    v &= 0xFFFFFFFFull;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
}
static uint32_t compact2(uint64_t v)
{
    v &= 0x5555555555555555ull;
    v = (v | (v >> 1)) & 0x3333333333333333ull;
    v = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
    v = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
    v = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
    return (uint32_t)v;
}
static uint64_t spread3(uint64_t v) /* two zeros between bits, 21 bits */
{
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x001F00000000FFFFull;
    v = (v | (v << 16)) & 0x001F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
static uint32_t compact3(uint64_t v)
{
    v &= 0x1249249249249249ull;
    v = (v | (v >> 2)) & 0x10C30C30C30C30C3ull;
    v = (v | (v >> 4)) & 0x100F00F00F00F00Full;
    v = (v | (v >> 8)) & 0x001F0000FF0000FFull;
    v = (v | (v >> 16)) & 0x001F00000000FFFFull;
    v = (v | (v >> 32)) & 0x00000000001FFFFFull;
    return (uint32_t)v;
}

/* morton_id::encode, morton_id.hpp:132-140 (2D), 350-359 (3D). */
uint64_t oracle_encode(int rank, int depth, const uint32_t* c, int level)
{
    (void)depth;
    uint64_t m;
    if (rank == 2)
        m = spread2(c[0]) | (spread2(c[1]) << 1);
    else
        m = spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
    return (m << 6) | ((uint64_t)level & 0x3F);
}

/* morton_id::decode, morton_id.hpp:118-130, 334-348. */
void oracle_decode(int rank, uint64_t id, uint32_t* c, int* level)
{
    *level = (int)(id & 0x3F);
    const uint64_t m = id >> 6;
    if (rank == 2) {
        c[0] = compact2(m);
        c[1] = compact2(m >> 1);
    } else {
        c[0] = compact3(m);
        c[1] = compact3(m >> 1);
        c[2] = compact3(m >> 2);
    }
}

/* morton_id::child_of = offset(id + 1, off), morton_id.hpp:64-83, 142-148. */
uint64_t oracle_child_of(int rank, int depth, uint64_t id, int off)
{
    uint32_t c[3];
    int      level;
    oracle_decode(rank, id + 1, c, &level);
    const uint32_t delta = 1u << (depth - level);
    c[0] += (uint32_t)(off & 1) * delta;
    c[1] += (uint32_t)((off >> 1) & 1) * delta;
    if (rank == 3) c[2] += (uint32_t)((off >> 2) & 1) * delta;
    return oracle_encode(rank, depth, c, level);
}

/* morton_id::parent_of, morton_id.hpp:103-116, 319-332. */
uint64_t oracle_parent_of(int rank, int depth, uint64_t id)
{
    uint32_t c[3];
    int      level;
    oracle_decode(rank, id, c, &level);
    const uint32_t off = 1u << (depth - level);
    for (int k = 0; k < rank; ++k) c[k] &= ~off;
    return oracle_encode(rank, depth, c, level - 1);
}

static int level_of(uint64_t id) { return (int)(id & 0x3F); }

/* ------------------------------------------------------------ hash map */
/* Morton id -> linear index (the reference's std::unordered_map m_index_map,
 * ndtree.hpp:2123).  Open addressing with tombstones. */
typedef struct {
    uint64_t* keys;
    size_t*   vals;
    uint8_t*  state; /* 0 empty, 1 full, 2 deleted */
    size_t    cap;   /* power of two */
    size_t    count;
} idmap;

static void map_init(idmap* m, size_t min_cap)
{
    size_t c = 16;
    while (c < 2 * min_cap + 16) c <<= 1;
    m->cap   = c;
    m->count = 0;
    m->keys  = (uint64_t*)calloc(c, sizeof(uint64_t));
    m->vals  = (size_t*)calloc(c, sizeof(size_t));
    m->state = (uint8_t*)calloc(c, 1);
}
static void map_free(idmap* m)
{
    free(m->keys);
    free(m->vals);
    free(m->state);
}
static void map_clear(idmap* m)
{
    memset(m->state, 0, m->cap);
    m->count = 0;
}
static size_t map_slot(const idmap* m, uint64_t k) { return (size_t)mix64(k) & (m->cap - 1); }
static long map_find(const idmap* m, uint64_t k)
{
    size_t s = map_slot(m, k);
    for (size_t n = 0; n < m->cap; ++n, s = (s + 1) & (m->cap - 1)) {
        if (m->state[s] == 0) return -1;
        if (m->state[s] == 1 && m->keys[s] == k) return (long)s;
    }
    return -1;
}
static void map_put(idmap* m, uint64_t k, size_t v)
{
    long f = map_find(m, k);
    if (f >= 0) {
        m->vals[f] = v;
        return;
    }
    size_t s = map_slot(m, k);
    while (m->state[s] == 1) s = (s + 1) & (m->cap - 1);
    m->state[s] = 1;
    m->keys[s]  = k;
    m->vals[s]  = v;
    m->count++;
}
static void map_erase(idmap* m, uint64_t k)
{
    long f = map_find(m, k);
    if (f >= 0) {
        m->state[f] = 2;
        m->count--;
    }
}

/* --------------------------------------------------------------- tree */
struct oracle_tree {
    int    rank, n, h, depth, nd, nf, ndir, nvar;
    double lengths[3]; /* physics_system's Domain_Sizes per Morton axis */
    size_t cap, size, flat, pad1, pstride; /* pstride = nvar * flat: fields of a patch, contiguous */
    uint64_t*        ids;      /* m_linear_index_map  ndtree.hpp:2149 */
    oracle_neighbor* nb;       /* m_neighbors         ndtree.hpp:2152 */
    int8_t*          status;   /* m_refine_status_buffer ndtree.hpp:2151 */
    double*          cur;      /* m_data_buffers      ndtree.hpp:2124 */
    double*          nxt;      /* m_next_buffers      ndtree.hpp:2125 */
    idmap            map;
    uint64_t*        to_refine;
    size_t           n_refine;
    uint64_t*        to_coarsen;
    size_t           n_coarsen;
    uint8_t*         refine_mark; /* membership of to_refine, by linear index */
    double*          scratch;
    size_t*          perm;
    int              fail;
};

static int g_threads = 0;
void oracle_set_threads(int n) { g_threads = n; }

static size_t ipow(size_t b, int e)
{
    size_t r = 1;
    while (e-- > 0) r *= b;
    return r;
}

static oracle_neighbor nb_none(void)
{
    oracle_neighbor x;
    memset(&x, 0, sizeof x);
    return x;
}
static oracle_neighbor nb_same(uint64_t id)
{
    oracle_neighbor x = nb_none();
    x.kind            = NB_SAME;
    x.ids[0]          = id;
    return x;
}

static void append(oracle_tree* t, uint64_t id, const oracle_neighbor* arr)
{
    /* ndtree::append, ndtree.hpp:1304-1316 */
    t->ids[t->size] = id;
    map_put(&t->map, id, t->size);
    memcpy(&t->nb[t->size * t->ndir], arr, sizeof(oracle_neighbor) * (size_t)t->ndir);
    t->size++;
}

oracle_tree* oracle_create(int rank, int n, int halo, int depth, size_t capacity)
{
    return oracle_create_fields(rank, n, halo, depth, capacity, 1);
}

oracle_tree* oracle_create_fields(int rank, int n, int halo, int depth, size_t capacity, int nvar)
{
    if ((rank != 2 && rank != 3) || n < 2 * halo || n % 2 || halo < 1 || nvar < 1) return NULL;
    oracle_tree* t = (oracle_tree*)calloc(1, sizeof *t);
    t->rank = rank;
    t->n    = n;
    t->h    = halo;
    t->depth = depth;
    t->nd   = 1 << rank;
    t->nf   = 1 << (rank - 1);
    t->ndir = 2 * rank;
    t->cap  = capacity;
    t->pad1 = (size_t)(n + 2 * halo);
    t->flat = ipow(t->pad1, rank);
    t->nvar    = nvar;
    t->pstride = t->flat * (size_t)nvar;
    t->lengths[0] = t->lengths[1] = t->lengths[2] = 1.0;
    t->ids  = (uint64_t*)calloc(capacity, sizeof(uint64_t));
    t->nb   = (oracle_neighbor*)calloc(capacity * (size_t)t->ndir, sizeof(oracle_neighbor));
    t->status = (int8_t*)calloc(capacity, 1);
    t->cur  = (double*)calloc(capacity * t->pstride, sizeof(double));
    t->nxt  = (double*)calloc(capacity * t->pstride, sizeof(double));
    t->to_refine  = (uint64_t*)malloc(capacity * sizeof(uint64_t));
    t->to_coarsen = (uint64_t*)malloc(capacity * sizeof(uint64_t));
    t->refine_mark = (uint8_t*)calloc(capacity, 1);
    t->scratch = (double*)malloc(t->pstride * sizeof(double));
    t->perm    = (size_t*)malloc(capacity * sizeof(size_t));
    map_init(&t->map, capacity);
    /* root with periodic self-neighbours, ndtree.hpp:411-421 */
    oracle_neighbor root[6];
    for (int d = 0; d < t->ndir; ++d) root[d] = nb_same(0);
    append(t, 0, root);
    return t;
}

void oracle_destroy(oracle_tree* t)
{
    if (!t) return;
    free(t->ids);
    free(t->nb);
    free(t->status);
    free(t->cur);
    free(t->nxt);
    free(t->to_refine);
    free(t->to_coarsen);
    free(t->refine_mark);
    free(t->scratch);
    free(t->perm);
    map_free(&t->map);
    free(t);
}

size_t oracle_size(const oracle_tree* t) { return t->size; }
size_t oracle_flat(const oracle_tree* t) { return t->flat; }
void oracle_get_ids(const oracle_tree* t, uint64_t* out)
{
    memcpy(out, t->ids, t->size * sizeof(uint64_t));
}
void oracle_get_neighbors(const oracle_tree* t, oracle_neighbor* out)
{
    memcpy(out, t->nb, t->size * (size_t)t->ndir * sizeof(oracle_neighbor));
}
void oracle_get_state(const oracle_tree* t, double* out)
{
    memcpy(out, t->cur, t->size * t->pstride * sizeof(double));
}
void oracle_set_state(oracle_tree* t, const double* in)
{
    memcpy(t->cur, in, t->size * t->pstride * sizeof(double));
}
int oracle_nvar(const oracle_tree* t) { return t->nvar; }

/* ------------------------------------------------- neighbour utilities */
/* Hypercube multi-index of a child offset, row-major with layout dim 0
 * slowest (neighbor.hpp:287-300 with container layout rules); offset
 * i = x + 2y (+ 4z) so the last layout dim carries x. */
static void child_coords(const oracle_tree* t, int i, int* c)
{
    c[0] = c[1] = c[2] = 0;
    for (int k = 0; k < t->rank; ++k) c[k] = (i >> (t->rank - 1 - k)) & 1;
}
static int child_linear(const oracle_tree* t, const int* c)
{
    int i = 0;
    for (int k = 0; k < t->rank; ++k) i |= c[k] << (t->rank - 1 - k);
    return i;
}
static int dir_dim(int d) { return d / 2; }
static int dir_pos(int d) { return d % 2; }
static int dir_opposite(int d) { return dir_pos(d) ? d - 1 : d + 1; } /* neighbor.hpp:168-173 */

/* s_neighbor_relation_maps, neighbor.hpp:291-313: 1 = ParentNeighbor. */
static int is_parent_neighbor(const oracle_tree* t, int i, int d)
{
    int c[3];
    child_coords(t, i, c);
    return dir_pos(d) ? c[dir_dim(d)] == 1 : c[dir_dim(d)] == 0;
}

/* compute_fine_boundary_linear_index, neighbor.hpp:316-337 (dim 0 fastest). */
static int fine_boundary_index(const oracle_tree* t, const int* c, int normal)
{
    int lin = 0, mult = 1;
    for (int k = 0; k < t->rank; ++k) {
        if (k == normal) continue;
        lin += c[k] * mult;
        mult *= 2;
    }
    return lin;
}

/* compute_boundary_children, neighbor.hpp:397-417. */
static void boundary_children(const oracle_tree* t, int d, int* out)
{
    for (int i = 0; i < t->nd; ++i) {
        if (!is_parent_neighbor(t, i, d)) continue;
        int c[3];
        child_coords(t, i, c);
        out[fine_boundary_index(t, c, dir_dim(d))] = i;
    }
}

/* compute_contact_quadrant, neighbor.hpp:340-364. */
static void contact_quadrant(const oracle_tree* t, int k, int d, uint8_t* q)
{
    for (int i = 0; i < t->rank; ++i) {
        if (i == dir_dim(d))
            q[i] = dir_pos(d) ? 0 : 1;
        else {
            q[i] = (uint8_t)(k % 2);
            k /= 2;
        }
    }
}

/* compute_child_neighbors, neighbor.hpp:420-493. */
static void child_neighbors(const oracle_tree* t, uint64_t parent, const oracle_neighbor* pnb,
                            int i, oracle_neighbor* out)
{
    int c[3];
    child_coords(t, i, c);
    for (int d = 0; d < t->ndir; ++d) {
        if (!is_parent_neighbor(t, i, d) || parent == 0) {
            int sc[3] = { c[0], c[1], c[2] };
            sc[dir_dim(d)] = (sc[dir_dim(d)] + 1) % 2; /* get_sibling_offset :383-395 */
            out[d] = nb_same(oracle_child_of(t->rank, t->depth, parent, child_linear(t, sc)));
            continue;
        }
        const oracle_neighbor* p = &pnb[d];
        oracle_neighbor        r = nb_none();
        if (p->kind == NB_SAME) {
            r.kind   = NB_COARSER;
            r.ids[0] = p->ids[0];
            for (int k = 0; k < t->rank; ++k) r.quadrant[k] = (uint8_t)c[k];
            r.quadrant[dir_dim(d)] = dir_pos(d) ? 0 : 1; /* :367-379 */
        } else if (p->kind == NB_FINER) {
            r = nb_same(p->ids[fine_boundary_index(t, c, dir_dim(d))]);
        }
        out[d] = r; /* none and coarser parents give none */
    }
}

/* compute_parent_neighbors, neighbor.hpp:495-572. */
static void parent_neighbors(const oracle_tree* t, const oracle_neighbor* cnb, oracle_neighbor* out)
{
    for (int d = 0; d < t->ndir; ++d) {
        int bc[4];
        boundary_children(t, d, bc);
        const oracle_neighbor* first = &cnb[bc[0] * t->ndir + d];
        oracle_neighbor        r     = nb_none();
        if (first->kind == NB_SAME) {
            r.kind = NB_FINER;
            for (int i = 0; i < t->nf; ++i) {
                const oracle_neighbor* cn = &cnb[bc[i] * t->ndir + d];
                r.ids[i] = cn->kind == NB_SAME ? cn->ids[0] : 0;
            }
        } else if (first->kind == NB_COARSER) {
            r = nb_same(first->ids[0]);
        }
        out[d] = r;
    }
}

static size_t index_of(oracle_tree* t, uint64_t id, int* ok)
{
    long s = map_find(&t->map, id);
    if (s < 0) {
        *ok = 0;
        return 0;
    }
    return t->map.vals[s];
}

/* enforce_symmetry_after_refinement, ndtree.hpp:942-1037. */
static void symmetry_after_refinement(oracle_tree* t, uint64_t parent)
{
    int    ok  = 1;
    size_t pix = index_of(t, parent, &ok);
    oracle_neighbor pnb[6];
    memcpy(pnb, &t->nb[pix * t->ndir], sizeof(oracle_neighbor) * (size_t)t->ndir);
    for (int d = 0; d < t->ndir; ++d) {
        const int od = dir_opposite(d);
        int       bc[4];
        boundary_children(t, d, bc);
        if (pnb[d].kind == NB_SAME) {
            oracle_neighbor nn = nb_none();
            nn.kind            = NB_FINER;
            for (int i = 0; i < t->nf; ++i)
                nn.ids[i] = oracle_child_of(t->rank, t->depth, parent, bc[i]);
            size_t ni = index_of(t, pnb[d].ids[0], &ok);
            if (!ok) { t->fail = -2; return; }
            t->nb[ni * t->ndir + od] = nn;
        } else if (pnb[d].kind == NB_FINER) {
            for (int i = 0; i < t->nf; ++i) {
                size_t ni = index_of(t, pnb[d].ids[i], &ok);
                if (!ok) { t->fail = -2; return; }
                t->nb[ni * t->ndir + od] =
                    nb_same(oracle_child_of(t->rank, t->depth, parent, bc[i]));
            }
        }
    }
}

/* enforce_symmetry_after_recombining, ndtree.hpp:1039-1125. */
static void symmetry_after_recombining(oracle_tree* t, uint64_t parent, const oracle_neighbor* pnb)
{
    for (int d = 0; d < t->ndir; ++d) {
        const int od = dir_opposite(d);
        int       ok = 1;
        if (pnb[d].kind == NB_SAME) {
            size_t ni = index_of(t, pnb[d].ids[0], &ok);
            if (ok) t->nb[ni * t->ndir + od] = nb_same(parent);
        } else if (pnb[d].kind == NB_FINER) {
            for (int i = 0; i < t->nf; ++i) {
                size_t ni = index_of(t, pnb[d].ids[i], &ok);
                if (!ok) { /* m_index_map.at throws inside noexcept: the reference terminates */
                    t->fail = -3;
                    return;
                }
                oracle_neighbor nn = nb_none();
                nn.kind            = NB_COARSER;
                nn.ids[0]          = parent;
                contact_quadrant(t, i, od, nn.quadrant);
                t->nb[ni * t->ndir + od] = nn;
            }
        }
    }
}

/* ------------------------------------------------ inter-grid transfer */
/* patch_mapping_impl + interpolate_patch / restrict_patches,
 * ndtree.hpp:1463-1555; linear_interpolator, intergrid_operator.hpp:41-107.
 * fn(kind): 0 interpolate (parent at `a` -> children a2..), 1 restrict. */
static void intergrid_field(oracle_tree* t, size_t coarse, size_t fine_start, int restrict_mode, int field);
static void intergrid(oracle_tree* t, size_t coarse, size_t fine_start, int restrict_mode)
{
    /* every field of the cell type moves the same way (patch_mapping_impl
     * over the deconstructed map types, ndtree.hpp:1463-1497) */
    for (int f = 0; f < t->nvar; ++f) intergrid_field(t, coarse, fine_start, restrict_mode, f);
}
static void intergrid_field(oracle_tree* t, size_t coarse, size_t fine_start, int restrict_mode, int field)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const size_t s0 = rank == 2 ? P1 : P1 * P1, s1 = rank == 2 ? 1 : P1;
    const int    half = n / 2;
    double*      buf  = t->cur;
    int          idx[3];
    const int    lo = h, hi = n + h;
    for (idx[0] = lo; idx[0] < hi; ++idx[0])
        for (idx[1] = lo; idx[1] < hi; ++idx[1])
            for (idx[2] = (rank == 3 ? lo : 0); idx[2] < (rank == 3 ? hi : 1); ++idx[2]) {
                int    fc[3], base[3];
                size_t coarse_idx = 0, base_idx = 0;
                for (int d = 0; d < rank; ++d) {
                    fc[d]   = (idx[d] - h) / half;
                    base[d] = ((idx[d] - h) % half) * 2 + h;
                }
                const int child = child_linear(t, fc);
                if (rank == 2) {
                    coarse_idx = (size_t)idx[0] * P1 + (size_t)idx[1];
                    base_idx   = (size_t)base[0] * P1 + (size_t)base[1];
                } else {
                    coarse_idx = ((size_t)idx[0] * P1 + (size_t)idx[1]) * P1 + (size_t)idx[2];
                    base_idx   = ((size_t)base[0] * P1 + (size_t)base[1]) * P1 + (size_t)base[2];
                }
                double*       cp = buf + coarse * t->pstride + (size_t)field * t->flat;
                double*       fp = buf + (fine_start + (size_t)child) * t->pstride + (size_t)field * t->flat;
                /* hypercube_offset<layout,2> order: row-major, dim 0 slowest
                 * (patch_utils.hpp:203-234) */
                size_t off[8];
                int    k = 0;
                if (rank == 2) {
                    for (int a = 0; a < 2; ++a)
                        for (int b = 0; b < 2; ++b) off[k++] = base_idx + a * s0 + b * s1;
                } else {
                    for (int a = 0; a < 2; ++a)
                        for (int b = 0; b < 2; ++b)
                            for (int c = 0; c < 2; ++c)
                                off[k++] = base_idx + a * s0 + b * s1 + c;
                }
                if (restrict_mode) {
                    double sum = 0.0;
                    for (int q = 0; q < k; ++q) sum += fp[off[q]];
                    cp[coarse_idx] = sum / (double)k;
                } else {
                    for (int q = 0; q < k; ++q) fp[off[q]] = cp[coarse_idx];
                }
            }
}

/* ------------------------------------------------------------- cycle */
static int refine_eligible(const oracle_tree* t, size_t i)
{
    /* is_refine_elegible, ndtree.hpp:1888-1896 */
    return t->status[i] == ST_REFINE && level_of(t->ids[i]) < t->depth;
}

static int coarsen_eligible(oracle_tree* t, uint64_t parent)
{
    /* is_coarsen_elegible, ndtree.hpp:1899-1917 */
    for (int i = 0; i < t->nd; ++i) {
        int    ok  = 1;
        size_t idx = index_of(t, oracle_child_of(t->rank, t->depth, parent, i), &ok);
        if (!ok) return 0;
        if (t->status[idx] != ST_COARSEN) return 0;
    }
    return 1;
}

static int cmp_u64(const void* a, const void* b)
{
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* apply_refine_coarsen, ndtree.hpp:904-940. */
static void apply_refine_coarsen(oracle_tree* t)
{
    t->n_refine  = 0;
    t->n_coarsen = 0;
    uint64_t* parents = (uint64_t*)malloc((t->size + 1) * sizeof(uint64_t));
    size_t    np      = 0;
    for (size_t i = 0; i < t->size; ++i) {
        if (t->ids[i] == 0) continue;
        parents[np++] = oracle_parent_of(t->rank, t->depth, t->ids[i]);
    }
    qsort(parents, np, sizeof(uint64_t), cmp_u64);
    size_t u = 0;
    for (size_t i = 0; i < np; ++i)
        if (u == 0 || parents[u - 1] != parents[i]) parents[u++] = parents[i];
    for (size_t i = 0; i < t->size; ++i)
        if (refine_eligible(t, i)) t->to_refine[t->n_refine++] = t->ids[i];
    for (size_t i = 0; i < u; ++i)
        if (coarsen_eligible(t, parents[i])) t->to_coarsen[t->n_coarsen++] = parents[i];
    free(parents);
}

static int cmp_level_desc(const void* a, const void* b)
{
    const int la = level_of(*(const uint64_t*)a), lb = level_of(*(const uint64_t*)b);
    return lb - la;
}

/* balancing, ndtree.hpp:1127-1240. Membership of m_to_refine (the reference
 * searches the vector linearly) is kept in a per-leaf mark array. */
static void balancing(oracle_tree* t)
{
    int ok = 1;
    memset(t->refine_mark, 0, t->size);
    for (size_t i = 0; i < t->n_refine; ++i) t->refine_mark[index_of(t, t->to_refine[i], &ok)] = 1;
    for (size_t i = 0; i < t->n_refine; ++i) {
        const size_t ix = index_of(t, t->to_refine[i], &ok);
        for (int d = 0; d < t->ndir; ++d) {
            const oracle_neighbor* nb = &t->nb[ix * t->ndir + d];
            if (nb->kind != NB_COARSER) continue;
            const size_t cx = index_of(t, nb->ids[0], &ok);
            if (!t->refine_mark[cx]) {
                t->refine_mark[cx]             = 1;
                t->to_refine[t->n_refine++]    = nb->ids[0];
            }
        }
    }
    /* sort by level, descending; the reference's std::ranges::sort is not
     * stable, and nothing downstream depends on the order within a level. */
    qsort(t->to_refine, t->n_refine, sizeof(uint64_t), cmp_level_desc);

    size_t keep = 0;
    for (size_t i = 0; i < t->n_coarsen; ++i) {
        const uint64_t parent = t->to_coarsen[i];
        int            veto   = 0;
        for (int d = 0; d < t->ndir && !veto; ++d) {
            int bc[4];
            boundary_children(t, d, bc);
            for (int j = 0; j < t->nf && !veto; ++j) {
                const uint64_t c  = oracle_child_of(t->rank, t->depth, parent, bc[j]);
                const size_t   cx = index_of(t, c, &ok);
                const oracle_neighbor* nb = &t->nb[cx * t->ndir + d];
                if (nb->kind == NB_FINER) veto = 1;
                else if (nb->kind == NB_SAME) {
                    int    ok2 = 1;
                    size_t sx  = index_of(t, nb->ids[0], &ok2);
                    if (ok2 && t->refine_mark[sx]) veto = 1;
                }
            }
        }
        if (!veto) t->to_coarsen[keep++] = parent;
    }
    t->n_coarsen = keep;
}

/* fragment(node), ndtree.hpp:727-778. */
static void fragment_one(oracle_tree* t, uint64_t node)
{
    int    ok   = 1;
    size_t from = index_of(t, node, &ok);
    const size_t start_to = t->size;
    oracle_neighbor pnb[6];
    memcpy(pnb, &t->nb[from * t->ndir], sizeof(oracle_neighbor) * (size_t)t->ndir);
    for (int i = 0; i < t->nd; ++i) {
        oracle_neighbor arr[6];
        child_neighbors(t, node, pnb, i, arr);
        append(t, oracle_child_of(t->rank, t->depth, node, i), arr);
    }
    symmetry_after_refinement(t, node);
    intergrid(t, from, start_to, 0);
    map_erase(&t->map, node);
}

/* recombine(parent), ndtree.hpp:780-834. */
static void recombine_one(oracle_tree* t, uint64_t parent)
{
    int             ok = 1;
    const size_t    start = index_of(t, oracle_child_of(t->rank, t->depth, parent, 0), &ok);
    oracle_neighbor cnb[8 * 6];
    for (int i = 0; i < t->nd; ++i) {
        const uint64_t c  = oracle_child_of(t->rank, t->depth, parent, i);
        const size_t   cx = index_of(t, c, &ok);
        memcpy(&cnb[i * t->ndir], &t->nb[cx * t->ndir], sizeof(oracle_neighbor) * (size_t)t->ndir);
        map_erase(&t->map, c);
    }
    oracle_neighbor pnb[6];
    parent_neighbors(t, cnb, pnb);
    const size_t to = t->size;
    append(t, parent, pnb);
    intergrid(t, to, start, 1);
    symmetry_after_recombining(t, parent, pnb);
}

static void swap_entries(oracle_tree* t, size_t i, size_t j)
{
    /* block_buffer_swap, ndtree.hpp:1980-2001 */
    if (i == j) return;
    uint64_t ti = t->ids[i];
    t->ids[i]   = t->ids[j];
    t->ids[j]   = ti;
    int8_t s     = t->status[i];
    t->status[i] = t->status[j];
    t->status[j] = s;
    oracle_neighbor tmp[6];
    memcpy(tmp, &t->nb[i * t->ndir], sizeof(oracle_neighbor) * (size_t)t->ndir);
    memcpy(&t->nb[i * t->ndir], &t->nb[j * t->ndir], sizeof(oracle_neighbor) * (size_t)t->ndir);
    memcpy(&t->nb[j * t->ndir], tmp, sizeof(oracle_neighbor) * (size_t)t->ndir);
    memcpy(t->scratch, &t->cur[i * t->pstride], t->pstride * sizeof(double));
    memcpy(&t->cur[i * t->pstride], &t->cur[j * t->pstride], t->pstride * sizeof(double));
    memcpy(&t->cur[j * t->pstride], t->scratch, t->pstride * sizeof(double));
}

/* compact, ndtree.hpp:1919-1948. */
static void compact(oracle_tree* t)
{
    size_t tail = 0;
    for (size_t head = 0; head < t->size; ++head) {
        if (map_find(&t->map, t->ids[head]) >= 0) {
            swap_entries(t, head, tail);
            ++tail;
        }
    }
    t->size = tail;
    map_clear(&t->map);
    for (size_t i = 0; i < t->size; ++i) map_put(&t->map, t->ids[i], i);
}

static const uint64_t* g_sort_keys;
static int cmp_perm(const void* a, const void* b)
{
    return cmp_u64(&g_sort_keys[*(const size_t*)a], &g_sort_keys[*(const size_t*)b]);
}

/* sort_buffers, ndtree.hpp:1335-1414 (ids are unique, so any sort gives
 * the same permutation). */
static void sort_buffers(oracle_tree* t)
{
    for (size_t i = 0; i < t->size; ++i) t->perm[i] = i;
    g_sort_keys = t->ids;
    qsort(t->perm, t->size, sizeof(size_t), cmp_perm);
    uint64_t*        ids = (uint64_t*)malloc(t->size * sizeof(uint64_t));
    int8_t*          st  = (int8_t*)malloc(t->size);
    oracle_neighbor* nb  = (oracle_neighbor*)malloc(t->size * (size_t)t->ndir * sizeof(oracle_neighbor));
    for (size_t i = 0; i < t->size; ++i) {
        const size_t s = t->perm[i];
        ids[i]         = t->ids[s];
        st[i]          = t->status[s];
        memcpy(&nb[i * t->ndir], &t->nb[s * t->ndir], sizeof(oracle_neighbor) * (size_t)t->ndir);
        memcpy(&t->nxt[i * t->pstride], &t->cur[s * t->pstride], t->pstride * sizeof(double));
    }
    memcpy(t->ids, ids, t->size * sizeof(uint64_t));
    memcpy(t->status, st, t->size);
    memcpy(t->nb, nb, t->size * (size_t)t->ndir * sizeof(oracle_neighbor));
    memcpy(t->cur, t->nxt, t->size * t->pstride * sizeof(double));
    free(ids);
    free(st);
    free(nb);
    map_clear(&t->map);
    for (size_t i = 0; i < t->size; ++i) map_put(&t->map, t->ids[i], i);
}

/* reconstruct_tree, ndtree.hpp:1249-1271; flags replace update_refine_flags
 * (:886-902), which only fills m_refine_status_buffer. */
int oracle_reconstruct(oracle_tree* t, const int8_t* flags)
{
    t->fail = 0;
    memcpy(t->status, flags, t->size);
    apply_refine_coarsen(t);
    if (t->n_refine == 0 && t->n_coarsen == 0) return 0;
    balancing(t);
    if (t->n_refine == 0 && t->n_coarsen == 0) return 0;
    const size_t grow = t->n_refine * (size_t)t->nd + t->n_coarsen;
    if (t->size + grow > t->cap) return -1; /* the reference writes past its malloc here */
    for (size_t i = t->n_refine; i > 0; --i) {
        fragment_one(t, t->to_refine[i - 1]); /* coarsest first, ndtree.hpp:855-858 */
        if (t->fail) return t->fail;
    }
    for (size_t i = 0; i < t->n_coarsen; ++i) {
        recombine_one(t, t->to_coarsen[i]);
        if (t->fail) return t->fail;
    }
    compact(t);
    sort_buffers(t);
    return 0;
}

void oracle_refine_all(oracle_tree* t, int levels)
{
    for (int l = 0; l < levels; ++l) {
        int8_t* f = (int8_t*)malloc(t->size);
        memset(f, ST_REFINE, t->size);
        oracle_reconstruct(t, f);
        free(f);
        oracle_halo_exchange(t);
    }
}

/* ------------------------------------------------------- halo exchange */
/* halo_apply over all directions, patch_utils.hpp:162-251; per relation
 * same_t :315-332, finer_t :334-386, coarser_t :388-441; boundary: no-op
 * (:303-313). Face ghost slabs only (patch_layout.hpp:183-221). */
static void halo_one_field(oracle_tree* t, size_t i, int field);
static void halo_one(oracle_tree* t, size_t i)
{
    /* every field of the cell type (halo_exchange_update loops over the map
     * types, ndtree.hpp:1581-1596) */
    for (int f = 0; f < t->nvar; ++f) halo_one_field(t, i, f);
}
static void halo_one_field(oracle_tree* t, size_t i, int field)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const size_t fo = (size_t)field * t->flat;
    double*      self = t->cur + i * t->pstride + fo;
    for (int d = 0; d < t->ndir; ++d) {
        const oracle_neighbor* nb = &t->nb[i * t->ndir + d];
        if (nb->kind == NB_NONE) continue;
        const int dim = dir_dim(d), pos = dir_pos(d);
        int       lo[3], hi[3], idx[3] = { 0, 0, 0 };
        for (int k = 0; k < 3; ++k) {
            lo[k] = 0;
            hi[k] = 1;
        }
        for (int k = 0; k < rank; ++k) {
            if (k != dim) {
                lo[k] = h;
                hi[k] = n + h;
            } else {
                lo[k] = pos ? n + h : 0;
                hi[k] = pos ? n + 2 * h : h;
            }
        }
        const double* other[4] = { 0, 0, 0, 0 };
        int           ok       = 1;
        if (nb->kind == NB_SAME || nb->kind == NB_COARSER)
            other[0] = t->cur + index_of(t, nb->ids[0], &ok) * t->pstride + fo;
        else
            for (int k = 0; k < t->nf; ++k) other[k] = t->cur + index_of(t, nb->ids[k], &ok) * t->pstride + fo;
        for (idx[0] = lo[0]; idx[0] < hi[0]; ++idx[0])
            for (idx[1] = lo[1]; idx[1] < hi[1]; ++idx[1])
                for (idx[2] = lo[2]; idx[2] < hi[2]; ++idx[2]) {
                    size_t to = 0;
                    for (int k = 0; k < rank; ++k) to = to * P1 + (size_t)idx[k];
                    if (nb->kind == NB_SAME) {
                        int from[3] = { idx[0], idx[1], idx[2] };
                        from[dim] += pos ? -n : n;
                        size_t f = 0;
                        for (int k = 0; k < rank; ++k) f = f * P1 + (size_t)from[k];
                        self[to] = other[0][f];
                    } else if (nb->kind == NB_FINER) {
                        int base[3] = { idx[0], idx[1], idx[2] };
                        base[dim] += pos ? -n : n;
                        int fpi = 0, stride = 1;
                        for (int k = 0; k < rank; ++k) {
                            /* the reference takes the modulus with the normal
                             * dimension's size for every k (:357-359) */
                            base[k] = ((base[k] - h) * 2) % n + h;
                            if (k != dim) {
                                fpi += ((idx[k] - h) / (n / 2)) * stride;
                                stride *= 2;
                            }
                        }
                        size_t b = 0;
                        for (int k = 0; k < rank; ++k) b = b * P1 + (size_t)base[k];
                        const double* fp = other[fpi];
                        double        sum = 0.0;
                        if (rank == 2) {
                            sum += fp[b];
                            sum += fp[b + 1];
                            sum += fp[b + P1];
                            sum += fp[b + P1 + 1];
                            self[to] = sum / 4.0;
                        } else {
                            const size_t s0 = P1 * P1;
                            for (int a = 0; a < 2; ++a)
                                for (int bb = 0; bb < 2; ++bb)
                                    for (int c = 0; c < 2; ++c) sum += fp[b + a * s0 + bb * P1 + c];
                            self[to] = sum / 8.0;
                        }
                    } else { /* coarser */
                        int from[3] = { idx[0], idx[1], idx[2] };
                        from[dim] += pos ? -n : n;
                        for (int k = 0; k < rank; ++k) {
                            const int fine = from[k] - h;
                            from[k]        = h + nb->quadrant[k] * (n / 2) + fine / 2;
                        }
                        size_t f = 0;
                        for (int k = 0; k < rank; ++k) f = f * P1 + (size_t)from[k];
                        self[to] = other[0][f];
                    }
                }
    }
}

void oracle_halo_exchange(oracle_tree* t)
{
    /* halo_exchange_update_cpu, ndtree.hpp:1581-1596 */
    const long n = (long)t->size;
#pragma omp parallel for schedule(static) if (n > 64) num_threads(g_threads > 0 ? g_threads : 1)
    for (long i = 0; i < n; ++i) halo_one(t, (size_t)i);
}

/* ------------------------------------------------------------ geometry */
/* physics_system::cell_sizes, physics_system.hpp:58-85, unit domain. */
static void cell_sizes(const oracle_tree* t, uint64_t id, double* cs)
{
    const uint32_t psm = 1u << (t->depth - level_of(id));
    const double   maxc = (double)(1u << t->depth);
    for (int k = 0; k < t->rank; ++k) {
        const double patch = t->lengths[k] * (double)psm / maxc;
        cs[k]              = patch / (double)t->n;
    }
}

void oracle_set_lengths(oracle_tree* t, const double* lengths)
{
    for (int k = 0; k < t->rank; ++k) t->lengths[k] = lengths[k];
}

/* ------------------------------------------------------------- solver */
/* compute_time_step_cpu, amr_solver.hpp:355-413 (advection: the speed is
 * |v_d| for every cell, AdvectionPhysics.hpp:73-85). */
double oracle_compute_dt(const oracle_tree* t, const double* v, double cfl)
{
    double dt = 1.7976931348623157e308;
    for (size_t i = 0; i < t->size; ++i) {
        double cs[3];
        cell_sizes(t, t->ids[i], cs);
        for (int d = 0; d < t->rank; ++d) {
            const double speed = fabs(v[d]);
            if (speed > 1e-12) {
                const double c = cs[d] / speed;
                if (c < dt) dt = c;
            }
        }
    }
    return cfl * dt;
}

/* time_step_cpu, amr_solver.hpp:265-353, with AdvectionPhysics::rusanovFlux
 * (AdvectionPhysics.hpp:45-66) inlined term for term. */
static void time_step(oracle_tree* t, const double* v, double dt)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const size_t stride[3] = { 1, P1, P1 * P1 };
    const long   np = (long)t->size;
#pragma omp parallel for schedule(static) if (np > 16) num_threads(g_threads > 0 ? g_threads : 1)
    for (long pi = 0; pi < np; ++pi) {
        const size_t  p = (size_t)pi;
        double        cs[3];
        cell_sizes(t, t->ids[p], cs);
        const double* in  = t->cur + p * t->pstride;
        double*       out = t->nxt + p * t->pstride;
        int           idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    const double uc    = in[li];
                    double       total = 0.0;
                    for (int d = 0; d < rank; ++d) {
                        const double uL = in[li - stride[d]];
                        const double uR = in[li + stride[d]];
                        const double sp = fabs(v[d]);
                        const double fL = 0.5 * (uL * v[d] + uc * v[d]) - 0.5 * sp * (uc - uL);
                        const double fR = 0.5 * (uc * v[d] + uR * v[d]) - 0.5 * sp * (uR - uc);
                        const double dt_over_dx = dt / cs[d];
                        total -= dt_over_dx * (fR - fL);
                    }
                    out[li] = uc + total;
                }
    }
    /* swap_buffers, ndtree.hpp:1558-1579 */
    double* tmp = t->cur;
    t->cur      = t->nxt;
    t->nxt      = tmp;
    oracle_halo_exchange(t);
}

/* advance_batch_async (CPU branch), amr_solver.hpp:221-242. */
double oracle_advance(oracle_tree* t, size_t steps, const double* v, double cfl, double remaining,
                      size_t* executed)
{
    double acc   = 0.0;
    size_t count = 0;
    for (size_t s = 0; s < steps; ++s) {
        if (remaining <= 0.0) break;
        const double dt      = oracle_compute_dt(t, v, cfl);
        const double step_dt = dt < remaining ? dt : remaining;
        if (step_dt <= 0.0) break;
        time_step(t, v, step_dt);
        acc += step_dt;
        remaining -= step_dt;
        ++count;
    }
    if (executed) *executed = count;
    return acc;
}

/* ---------------------------------------------------------------- SSPRK */
/* The strong-stability-preserving Runge-Kutta integrators of the reference
 * (include/dg_helpers/time_integration/time.hpp:83-272, used there per
 * patch with a halo exchange before every stage, solver.hpp:162-244) applied
 * to the FV advection operator: the residual of a stage is
 *   R = -sum_d (F_R - F_L) / dx_d
 * with the Rusanov flux of AdvectionPhysics (as in time_step), and the
 * stage combinations are the reference's, operation for operation:
 *   stage 0           u* = u + R dt
 *   SSPRK2 stage 1    u' = ((u^n + u*) + R dt) * 0.5
 *   SSPRK3 stage 1    u2 = u^n * 0.75 + (u1 + R dt) * 0.25
 *   SSPRK3 stage 2    u' = u^n * (1/3) + (u2 + R dt) * (2/3)
 * mode: 0, 2, 31, 32 for the four forms.  Like the reference, which
 * combines whole padded containers, every cell of `out` is written (the
 * ghost cells with R = 0), and no halo exchange follows the last stage: the
 * next step starts with one (solver.hpp:174), and a criterion evaluated
 * between steps sees the combined ghosts, as in the reference. */
static void ssprk_stage(const oracle_tree* t, const double* v, double dt, int mode, const double* in,
                        const double* un, double* out)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const size_t stride[3] = { 1, P1, P1 * P1 };
    const long   np = (long)t->size;
#pragma omp parallel for schedule(static) if (np > 16) num_threads(g_threads > 0 ? g_threads : 1)
    for (long pi = 0; pi < np; ++pi) {
        const size_t p = (size_t)pi;
        double       cs[3];
        cell_sizes(t, t->ids[p], cs);
        const double* a = in + p * t->pstride;
        const double* b = un + p * t->pstride;
        double*       o = out + p * t->pstride;
        /* every cell of the padded patch, as the reference combines whole
         * containers; the residual is zero outside the interior */
        for (size_t li = 0; li < t->flat; ++li) {
            int    interior = 1;
            size_t r        = li;
            for (int k = 0; k < rank; ++k) {
                const size_t c = r % P1;
                r /= P1;
                if (c < (size_t)h || c >= (size_t)(n + h)) interior = 0;
            }
            const double uc = a[li];
            double       R  = 0.0;
            if (interior)
                for (int d = 0; d < rank; ++d) {
                    const double uL = a[li - stride[d]];
                    const double uR = a[li + stride[d]];
                    const double sp = fabs(v[d]);
                    const double fL = 0.5 * (uL * v[d] + uc * v[d]) - 0.5 * sp * (uc - uL);
                    const double fR = 0.5 * (uc * v[d] + uR * v[d]) - 0.5 * sp * (uR - uc);
                    R -= (fR - fL) / cs[d];
                }
            const double Rdt = R * dt;
            double       res;
            if (mode == 0) res = uc + Rdt;
            else if (mode == 2) res = (b[li] + uc + Rdt) * 0.5;
            else if (mode == 31) res = b[li] * 0.75 + (uc + Rdt) * 0.25;
            else res = b[li] * (1.0 / 3.0) + (uc + Rdt) * (2.0 / 3.0);
            o[li] = res;
        }
    }
}

/* halo exchange of an arbitrary state buffer of the tree */
static void halo_buffer(oracle_tree* t, double* buf)
{
    double* keep = t->cur;
    t->cur       = buf;
    oracle_halo_exchange(t);
    t->cur = keep;
}

/* advance_batch_async's loop (CFL step from compute_time_step_cpu, clamped to
 * the remaining time) with SSPRK2 (order 2) or SSPRK3 (order 3) steps. */
double oracle_ssprk_advance(oracle_tree* t, size_t steps, int order, const double* v, double cfl, double remaining,
                            size_t* executed)
{
    double* A = (double*)malloc((t->size > 0 ? t->size : 1) * t->pstride * sizeof(double));
    double  acc   = 0.0;
    size_t  count = 0;
    if (A) memset(A, 0, (t->size > 0 ? t->size : 1) * t->pstride * sizeof(double));
    for (size_t s = 0; A && s < steps; ++s) {
        if (remaining <= 0.0) break;
        const double dt      = oracle_compute_dt(t, v, cfl);
        const double step_dt = dt < remaining ? dt : remaining;
        if (step_dt <= 0.0) break;
        oracle_halo_exchange(t);
        if (order == 2) {
            ssprk_stage(t, v, step_dt, 0, t->cur, t->cur, A);
            halo_buffer(t, A);
            ssprk_stage(t, v, step_dt, 2, A, t->cur, t->nxt);
        } else {
            ssprk_stage(t, v, step_dt, 0, t->cur, t->cur, t->nxt);
            halo_buffer(t, t->nxt);
            ssprk_stage(t, v, step_dt, 31, t->nxt, t->cur, A);
            halo_buffer(t, A);
            ssprk_stage(t, v, step_dt, 32, A, t->cur, t->nxt);
        }
        double* tmp = t->cur;
        t->cur      = t->nxt;
        t->nxt      = tmp;
        acc += step_dt;
        remaining -= step_dt;
        ++count;
    }
    free(A);
    if (executed) *executed = count;
    return acc;
}

/* ------------------------------------------------------------ VTK file */
/* vtk_print::print (include/ndtree/vtk_print.hpp:53-257): legacy VTK,
 * BINARY (big-endian), DATASET UNSTRUCTURED_GRID with one quad (2D, type 9)
 * or voxel (3D, type 11) per interior cell; corner coordinates from
 * physics_system::patch_coord / cell_sizes (physics_system.hpp:58-104) on the
 * tree's domain lengths; CELL_DATA cell_index, is_halo (the reference evaluates
 * is_halo_cell on the padded layout for linear indices 0 .. n^rank - 1 of
 * every patch, vtk_print.hpp:217-228) and the scalar field. */
static void put_be(FILE* f, const void* v, size_t n)
{
    unsigned char b[8];
    memcpy(b, v, n);
    for (size_t i = 0; i < n / 2; ++i) {
        const unsigned char x = b[i];
        b[i]                  = b[n - 1 - i];
        b[n - 1 - i]          = x;
    }
    fwrite(b, 1, n, f);
}
static void put_f64(FILE* f, double v) { put_be(f, &v, 8); }
static void put_i32(FILE* f, int v) { put_be(f, &v, 4); }

static int padded_is_halo(const oracle_tree* t, size_t li)
{
    size_t stride = 1;
    for (int k = 1; k < t->rank; ++k) stride *= t->pad1;
    for (int k = 0; k < t->rank; ++k) {
        const size_t rel = li / stride;
        if (rel < (size_t)t->h || rel >= t->pad1 - (size_t)t->h) return 1;
        li %= stride;
        stride /= t->pad1;
    }
    return 0;
}

int oracle_write_vtk(const oracle_tree* t, const char* path, const char* fields)
{
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t box = (size_t)1 << rank, per = ipow((size_t)n, rank), cells = t->size * per;
    const double maxc = (double)(1u << t->depth);
    fprintf(f, "# vtk DataFile Version 3.0\nAMR Tree Structure\nBINARY\nDATASET UNSTRUCTURED_GRID\n");
    fprintf(f, "POINTS %zu double\n", cells * box);
    for (size_t p = 0; p < t->size; ++p) {
        uint32_t c[3] = { 0, 0, 0 };
        int      level;
        oracle_decode(rank, t->ids[p], c, &level);
        double origin[3], cs[3];
        for (int k = 0; k < rank; ++k) {
            /* physics_system::patch_coord / patch_sizes (physics_system.hpp:58-97) */
            origin[k]         = t->lengths[k] * (double)c[k] / maxc;
            const double size = t->lengths[k] * (double)(1u << (t->depth - level)) / maxc;
            cs[k]             = size / (double)n;
        }
        int idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    if (rank == 2) {
                        const double x = origin[0] + (double)(idx[1] - h) * cs[0];
                        const double y = origin[1] + (double)(idx[0] - h) * cs[1];
                        const double X = x + cs[0], Y = y + cs[1];
                        put_f64(f, x); put_f64(f, y); put_f64(f, 0.0);
                        put_f64(f, X); put_f64(f, y); put_f64(f, 0.0);
                        put_f64(f, X); put_f64(f, Y); put_f64(f, 0.0);
                        put_f64(f, x); put_f64(f, Y); put_f64(f, 0.0);
                    } else {
                        const double x = origin[0] + (double)(idx[2] - h) * cs[0];
                        const double y = origin[1] + (double)(idx[1] - h) * cs[1];
                        const double z = origin[2] + (double)(idx[0] - h) * cs[2];
                        const double X = x + cs[0], Y = y + cs[1], Z = z + cs[2];
                        put_f64(f, x); put_f64(f, y); put_f64(f, z);
                        put_f64(f, X); put_f64(f, y); put_f64(f, z);
                        put_f64(f, x); put_f64(f, Y); put_f64(f, z);
                        put_f64(f, X); put_f64(f, Y); put_f64(f, z);
                        put_f64(f, x); put_f64(f, y); put_f64(f, Z);
                        put_f64(f, X); put_f64(f, y); put_f64(f, Z);
                        put_f64(f, x); put_f64(f, Y); put_f64(f, Z);
                        put_f64(f, X); put_f64(f, Y); put_f64(f, Z);
                    }
                }
    }
    fprintf(f, "CELLS %zu %zu\n", cells, cells * (box + 1));
    for (size_t i = 0; i < cells; ++i) {
        put_i32(f, (int)box);
        for (size_t j = 0; j < box; ++j) put_i32(f, (int)(i * box + j));
    }
    fprintf(f, "CELL_TYPES %zu\n", cells);
    for (size_t i = 0; i < cells; ++i) put_i32(f, rank == 2 ? 9 : 11);
    fprintf(f, "CELL_DATA %zu\nSCALARS cell_index int 1\nLOOKUP_TABLE default\n", cells);
    for (size_t i = 0; i < cells; ++i) put_i32(f, (int)i);
    fprintf(f, "SCALARS is_halo int 1\nLOOKUP_TABLE default\n");
    for (size_t p = 0; p < t->size; ++p)
        for (size_t j = 0; j < per; ++j) put_i32(f, padded_is_halo(t, j));
    /* one SCALARS block per field, in tuple order; `fields` names them,
     * separated by commas */
    const char* name = fields;
    for (int fi = 0; fi < t->nvar; ++fi) {
        size_t len = 0;
        while (name[len] && name[len] != ',') ++len;
        fprintf(f, "SCALARS %.*s double 1\nLOOKUP_TABLE default\n", (int)len, name);
        name += len + (name[len] == ',' ? 1 : 0);
        for (size_t p = 0; p < t->size; ++p) {
            const double* u = t->cur + p * t->pstride + (size_t)fi * t->flat;
            int           idx[3];
            for (idx[0] = h; idx[0] < n + h; ++idx[0])
                for (idx[1] = h; idx[1] < n + h; ++idx[1])
                    for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                        size_t li = 0;
                        for (int k = 0; k < rank; ++k) li = li * t->pad1 + (size_t)idx[k];
                        put_f64(f, u[li]);
                    }
        }
    }
    return fclose(f) == 0 ? 0 : -1;
}

/* ------------------------------------------------------------- adjoint */
/* Transpose of one oracle step (time_step: flux update on exchanged ghosts,
 * then the halo fill of the new state), written as a scatter from the
 * forward loops so it is independent of the GPU's gather form.  As a linear
 * map of the padded input, time_step's cell update is
 *   out = uc - sum_d k_d [0.5 (v-|v|) uR + |v| uc - 0.5 (v+|v|) uL],
 * k_d = dt / cs_d (the Rusanov flux of AdvectionPhysics.hpp:45-66 expanded),
 * and halo_one's ghost = copy / mean of 2^rank fine cells / injection.
 * lam_in: adjoint of the state after the step (interior cells; ghost entries
 * ignored); lam_out: adjoint of the state before it, interior cells, ghost
 * entries zero.  The initial state's ghosts are the halo fill of its
 * interior (oracle_init_state + oracle_halo_exchange), so the halo transpose
 * applies before every step, the first included. */
static void adjoint_step(oracle_tree* t, const double* v, double dt, const double* lam_in, double* lam_out)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const size_t stride[3] = { 1, P1, P1 * P1 };
    const long   np = (long)t->size;
    memset(lam_out, 0, t->size * t->flat * sizeof(double));
    /* flux update transposed: scatter within each padded patch */
#pragma omp parallel for schedule(static) if (np > 16) num_threads(g_threads > 0 ? g_threads : 1)
    for (long pi = 0; pi < np; ++pi) {
        const size_t  p = (size_t)pi;
        double        cs[3];
        cell_sizes(t, t->ids[p], cs);
        const double* li_in = lam_in + p * t->flat;
        double*       lo    = lam_out + p * t->flat;
        int           idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    const double w  = li_in[li];
                    double       cc = 1.0;
                    for (int d = 0; d < rank; ++d) {
                        const double k_d = dt / cs[d], sp = fabs(v[d]);
                        cc -= k_d * sp;
                        lo[li + stride[d]] += -k_d * 0.5 * (v[d] - sp) * w;
                        lo[li - stride[d]] += k_d * 0.5 * (v[d] + sp) * w;
                    }
                    lo[li] += cc * w;
                }
    }
    /* halo fill transposed: every face ghost passes its adjoint to the cells
     * it was filled from (halo_one's loops), then is cleared */
    for (size_t i = 0; i < t->size; ++i) {
        double* self = lam_out + i * t->flat;
        for (int d = 0; d < t->ndir; ++d) {
            const oracle_neighbor* nb = &t->nb[i * t->ndir + d];
            const int              dim = dir_dim(d), pos = dir_pos(d);
            int                    lo[3], hi[3], idx[3] = { 0, 0, 0 };
            for (int k = 0; k < 3; ++k) {
                lo[k] = 0;
                hi[k] = 1;
            }
            for (int k = 0; k < rank; ++k) {
                if (k != dim) {
                    lo[k] = h;
                    hi[k] = n + h;
                } else {
                    lo[k] = pos ? n + h : 0;
                    hi[k] = pos ? n + 2 * h : h;
                }
            }
            int     ok = 1;
            double* other[4] = { 0, 0, 0, 0 };
            if (nb->kind == NB_SAME || nb->kind == NB_COARSER)
                other[0] = lam_out + index_of(t, nb->ids[0], &ok) * t->flat;
            else if (nb->kind == NB_FINER)
                for (int k = 0; k < t->nf; ++k) other[k] = lam_out + index_of(t, nb->ids[k], &ok) * t->flat;
            for (idx[0] = lo[0]; idx[0] < hi[0]; ++idx[0])
                for (idx[1] = lo[1]; idx[1] < hi[1]; ++idx[1])
                    for (idx[2] = lo[2]; idx[2] < hi[2]; ++idx[2]) {
                        size_t to = 0;
                        for (int k = 0; k < rank; ++k) to = to * P1 + (size_t)idx[k];
                        const double gadj = self[to];
                        self[to]          = 0.0;
                        if (nb->kind == NB_NONE) continue;
                        if (nb->kind == NB_SAME) {
                            int from[3] = { idx[0], idx[1], idx[2] };
                            from[dim] += pos ? -n : n;
                            size_t f = 0;
                            for (int k = 0; k < rank; ++k) f = f * P1 + (size_t)from[k];
                            other[0][f] += gadj;
                        } else if (nb->kind == NB_FINER) {
                            int base[3] = { idx[0], idx[1], idx[2] };
                            base[dim] += pos ? -n : n;
                            int fpi = 0, str = 1;
                            for (int k = 0; k < rank; ++k) {
                                base[k] = ((base[k] - h) * 2) % n + h;
                                if (k != dim) {
                                    fpi += ((idx[k] - h) / (n / 2)) * str;
                                    str *= 2;
                                }
                            }
                            size_t b = 0;
                            for (int k = 0; k < rank; ++k) b = b * P1 + (size_t)base[k];
                            double* fp = other[fpi];
                            if (rank == 2) {
                                fp[b] += gadj / 4.0;
                                fp[b + 1] += gadj / 4.0;
                                fp[b + P1] += gadj / 4.0;
                                fp[b + P1 + 1] += gadj / 4.0;
                            } else {
                                const size_t s0 = P1 * P1;
                                for (int a = 0; a < 2; ++a)
                                    for (int bb = 0; bb < 2; ++bb)
                                        for (int c = 0; c < 2; ++c) fp[b + a * s0 + bb * P1 + c] += gadj / 8.0;
                            }
                        } else {
                            int from[3] = { idx[0], idx[1], idx[2] };
                            from[dim] += pos ? -n : n;
                            for (int k = 0; k < rank; ++k) {
                                const int fine = from[k] - h;
                                from[k]        = h + nb->quadrant[k] * (n / 2) + fine / 2;
                            }
                            size_t f = 0;
                            for (int k = 0; k < rank; ++k) f = f * P1 + (size_t)from[k];
                            other[0][f] += gadj;
                        }
                    }
        }
    }
}

/* Gradient of <lam_T, u_T> with respect to the interior of u_0 for
 * oracle_advance(steps, v, cfl, remaining) started from the tree's current
 * (frozen) mesh: the step sizes of the forward run, then the transposed
 * steps in reverse order.  Returns the number of executed steps. */
size_t oracle_adjoint(oracle_tree* t, size_t steps, const double* v, double cfl, double remaining,
                      const double* lam_T, double* lam_0)
{
    double* dts = (double*)malloc((steps ? steps : 1) * sizeof(double));
    size_t  ex  = 0;
    for (size_t s = 0; s < steps; ++s) { /* oracle_advance's step sizes */
        if (remaining <= 0.0) break;
        const double dt      = oracle_compute_dt(t, v, cfl);
        const double step_dt = dt < remaining ? dt : remaining;
        if (step_dt <= 0.0) break;
        dts[ex++] = step_dt;
        remaining -= step_dt;
    }
    const size_t bytes = t->size * t->flat * sizeof(double);
    double*      a     = (double*)malloc(bytes);
    double*      b     = (double*)malloc(bytes);
    memcpy(a, lam_T, bytes);
    /* ghost entries of the terminal adjoint are not part of the interior map */
    const int rank = t->rank, n = t->n, h = t->h;
    for (size_t i = 0; i < t->size * t->flat; ++i) {
        size_t r = i % t->flat;
        int    inside = 1;
        for (int k = rank - 1; k >= 0; --k) {
            const int c = (int)(r % t->pad1);
            r /= t->pad1;
            inside = inside && c >= h && c < n + h;
        }
        if (!inside) a[i] = 0.0;
    }
    for (size_t s = ex; s-- > 0;) {
        adjoint_step(t, v, dts[s], a, b);
        double* tmp = a;
        a           = b;
        b           = tmp;
    }
    memcpy(lam_0, a, bytes);
    free(a);
    free(b);
    free(dts);
    return ex;
}

/* ---------------------------------------------------------------- Euler */
/* EulerPhysics<DIM> (include/solver/EulerPhysics.hpp:17-170) with
 * amr_solver's time_step_cpu / compute_time_step_cpu / initialize
 * (amr_solver.hpp:105-145, 265-413): NVAR = DIM + 2 conservative fields
 * (rho, rho u_d, E), Rusanov flux with the maximum of |u_dir| + a of the two
 * sides, each face flux evaluated by both cells (as the reference does),
 * forward Euler. */
static double max_d(double a, double b) { return (a < b) ? b : a; } /* std::max */

static void euler_flux(int dim, const double* UL, const double* UR, double* flux, int dir, double gamma)
{
    const double inv_rho_L = 1.0 / UL[0];
    double       K_L       = 0.0;
    for (int d = 0; d < dim; ++d) K_L += UL[1 + d] * UL[1 + d];
    K_L *= 0.5 * inv_rho_L;
    const double p_L     = (gamma - 1.0) * (UL[dim + 1] - K_L);
    const double a_L     = sqrt(gamma * p_L * inv_rho_L);
    const double u_dir_L = UL[1 + dir] * inv_rho_L;
    const double inv_rho_R = 1.0 / UR[0];
    double       K_R       = 0.0;
    for (int d = 0; d < dim; ++d) K_R += UR[1 + d] * UR[1 + d];
    K_R *= 0.5 * inv_rho_R;
    const double p_R     = (gamma - 1.0) * (UR[dim + 1] - K_R);
    const double a_R     = sqrt(gamma * p_R * inv_rho_R);
    const double u_dir_R = UR[1 + dir] * inv_rho_R;
    const double smax    = max_d(fabs(u_dir_L) + a_L, fabs(u_dir_R) + a_R);
    flux[0] = 0.5 * (UL[1 + dir] + UR[1 + dir] - smax * (UR[0] - UL[0]));
    for (int d = 0; d < dim; ++d) {
        double fL_mom = UL[1 + d] * u_dir_L;
        double fR_mom = UR[1 + d] * u_dir_R;
        if (d == dir) {
            fL_mom += p_L;
            fR_mom += p_R;
        }
        flux[1 + d] = 0.5 * (fL_mom + fR_mom - smax * (UR[1 + d] - UL[1 + d]));
    }
    const double fL_E = u_dir_L * (UL[dim + 1] + p_L);
    const double fR_E = u_dir_R * (UR[dim + 1] + p_R);
    flux[dim + 1]     = 0.5 * (fL_E + fR_E - smax * (UR[dim + 1] - UL[dim + 1]));
}

/* getMaxSpeed: |u_dir| + a of one cell */
static double euler_speed(int dim, const double* U, int dir, double gamma)
{
    const double inv_rho = 1.0 / U[0];
    double       K       = 0.0;
    for (int d = 0; d < dim; ++d) K += U[1 + d] * U[1 + d];
    K *= 0.5 * inv_rho;
    const double p     = (gamma - 1.0) * (U[dim + 1] - K);
    const double a     = sqrt(gamma * p * inv_rho);
    const double u_dir = U[1 + dir] * inv_rho;
    return fabs(u_dir) + a;
}

static void gather_cell(const oracle_tree* t, const double* patch, size_t li, double* U)
{
    for (int f = 0; f < t->nvar; ++f) U[f] = patch[(size_t)f * t->flat + li];
}

double oracle_euler_dt(const oracle_tree* t, double gamma, double cfl)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const long   np = (long)t->size;
    double       dt = 1.7976931348623157e308;
    /* a minimum: the same value in any order (EXECUTION=PAR reduces in
     * parallel as well) */
#pragma omp parallel for schedule(static) reduction(min : dt) if (np > 16) num_threads(g_threads > 0 ? g_threads : 1)
    for (long pi = 0; pi < np; ++pi) {
        const size_t p = (size_t)pi;
        double       cs[3];
        cell_sizes(t, t->ids[p], cs);
        const double* u = t->cur + p * t->pstride;
        int           idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    double U[5];
                    gather_cell(t, u, li, U);
                    for (int d = 0; d < rank; ++d) {
                        const double speed = euler_speed(rank, U, d, gamma);
                        if (speed > 1e-12) {
                            const double c = cs[d] / speed;
                            if (c < dt) dt = c;
                        }
                    }
                }
    }
    return cfl * dt;
}

static void euler_step(oracle_tree* t, double gamma, double dt)
{
    const int    rank = t->rank, n = t->n, h = t->h, nv = t->nvar;
    const size_t P1 = t->pad1;
    const size_t stride[3] = { 1, P1, P1 * P1 };
    const long   np = (long)t->size;
#pragma omp parallel for schedule(static) if (np > 16) num_threads(g_threads > 0 ? g_threads : 1)
    for (long pi = 0; pi < np; ++pi) {
        const size_t  p = (size_t)pi;
        double        cs[3];
        cell_sizes(t, t->ids[p], cs);
        const double* in  = t->cur + p * t->pstride;
        double*       out = t->nxt + p * t->pstride;
        int           idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    double total[5] = { 0, 0, 0, 0, 0 }, Uc[5], UL[5], UR[5], fL[5], fR[5];
                    gather_cell(t, in, li, Uc);
                    for (int d = 0; d < rank; ++d) {
                        gather_cell(t, in, li - stride[d], UL);
                        gather_cell(t, in, li + stride[d], UR);
                        euler_flux(rank, UL, Uc, fL, d, gamma);
                        euler_flux(rank, Uc, UR, fR, d, gamma);
                        const double dt_over_dx = dt / cs[d];
                        for (int k = 0; k < nv; ++k) total[k] -= dt_over_dx * (fR[k] - fL[k]);
                    }
                    for (int k = 0; k < nv; ++k) out[(size_t)k * t->flat + li] = in[(size_t)k * t->flat + li] + total[k];
                }
    }
    double* tmp = t->cur;
    t->cur      = t->nxt;
    t->nxt      = tmp;
    oracle_halo_exchange(t);
}

/* advance_batch_async (CPU branch) with EulerPhysics; fills dts (if not
 * NULL, room for `steps`) with the step sizes. */
double oracle_euler_advance(oracle_tree* t, size_t steps, double gamma, double cfl, double remaining,
                            size_t* executed, double* dts)
{
    double acc   = 0.0;
    size_t count = 0;
    for (size_t s = 0; s < steps; ++s) {
        if (remaining <= 0.0) break;
        const double dt      = oracle_euler_dt(t, gamma, cfl);
        const double step_dt = dt < remaining ? dt : remaining;
        if (step_dt <= 0.0) break;
        euler_step(t, gamma, step_dt);
        if (dts) dts[count] = step_dt;
        acc += step_dt;
        remaining -= step_dt;
        ++count;
    }
    if (executed) *executed = count;
    return acc;
}

/* amr_solver::initialize with the acoustic pulse of
 * benchmark/bench_fvm_solver_integration.b.cpp:140-178: primitive state
 * (rho_bg + 0.2 A e, 0, .., p_bg + A e), e = exp(-|x - c|^2 / width_sq),
 * converted by primitiveToConservative at each cell centre
 * (physics_system::cell_coord + 0.5 cell size). */
void oracle_euler_init_pulse(oracle_tree* t, double gamma, double rho_bg, double p_bg, double amplitude,
                             double width_sq, const double* centre)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const double maxc = (double)(1u << t->depth);
    for (size_t p = 0; p < t->size; ++p) {
        uint32_t mc[3];
        int      level;
        oracle_decode(rank, t->ids[p], mc, &level);
        double cs[3], origin[3];
        cell_sizes(t, t->ids[p], cs);
        for (int k = 0; k < rank; ++k) origin[k] = t->lengths[k] * (double)mc[k] / maxc;
        double* u = t->cur + p * t->pstride;
        int     idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    double x[3];
                    for (int k = 0; k < rank; ++k) {
                        const double cell = origin[k] + (double)(idx[rank - 1 - k] - h) * cs[k];
                        x[k]              = cell + 0.5 * cs[k];
                    }
                    double r_sq = 0.0;
                    for (int k = 0; k < rank; ++k) {
                        const double dx = x[k] - centre[k];
                        r_sq += dx * dx;
                    }
                    const double pert = amplitude * exp(-r_sq / width_sq);
                    const double rho  = rho_bg + (pert * 0.2);
                    const double pres = p_bg + pert;
                    /* primitiveToConservative (EulerPhysics.hpp:34-60), u = 0 */
                    double vel_squared = 0.0;
                    u[li] = rho;
                    for (int d = 0; d < rank; ++d) {
                        const double ud                        = 0.0;
                        u[(size_t)(1 + d) * t->flat + li] = rho * ud;
                        vel_squared += ud * ud;
                    }
                    u[(size_t)(rank + 1) * t->flat + li] = pres / (gamma - 1.0) + 0.5 * rho * vel_squared;
                }
    }
}

/* ------------------------------------------------------------ criteria */
/* max|grad u|*h with central differences over face ghosts and the any/all
 * patch rule of dg_helpers/globals/amr_indicators.hpp:186-225; level bounds
 * as in benchmark/bench_fvm_solver_integration_active_amr.b.cpp:92-102. */
void oracle_flags_gradient(const oracle_tree* t, double rthr, double cthr, int min_level,
                           int max_level, int8_t* out)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const size_t stride[3] = { 1, P1, P1 * P1 };
    for (size_t p = 0; p < t->size; ++p) {
        const double* u = t->cur + p * t->pstride;
        int any = 0, all = 1, idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    double s = 0.0;
                    for (int d = 0; d < rank; ++d) {
                        const double g = 0.5 * (u[li + stride[d]] - u[li - stride[d]]);
                        s += g * g;
                    }
                    const double val = sqrt(s);
                    if (val > rthr) any = 1;
                    if (!(val < cthr)) all = 0;
                }
        const int level = level_of(t->ids[p]);
        out[p] = (level < max_level && any) ? ST_REFINE
                 : (level > min_level && all) ? ST_COARSEN
                                              : ST_STABLE;
    }
}

/* Max-value rule over the padded patch, tests/advection_equation_amr.t.cpp:155-170. */
void oracle_flags_max(const oracle_tree* t, double rthr, double cthr, int min_level, int max_level,
                      int8_t* out)
{
    for (size_t p = 0; p < t->size; ++p) {
        const double* u = t->cur + p * t->pstride; /* the first field (e.g. Rho) */
        double        m = 0.0;
        for (size_t c = 0; c < t->flat; ++c)
            if (u[c] > m) m = u[c];
        const int level = level_of(t->ids[p]);
        out[p] = (m > rthr && level < max_level) ? ST_REFINE
                 : (m < cthr && level > min_level) ? ST_COARSEN
                                                   : ST_STABLE;
    }
}

void oracle_flags_random(const oracle_tree* t, uint64_t seed, uint64_t pass, double pr, double pc,
                         int min_level, int max_level, int8_t* out)
{
    for (size_t p = 0; p < t->size; ++p) {
        const uint64_t id    = t->ids[p];
        const int      level = level_of(id);
        int8_t         s     = ST_STABLE;
        if (oracle_unit_hash(seed, pass, id) < pr && level < max_level)
            s = ST_REFINE;
        else if (level > 0) {
            const uint64_t parent = oracle_parent_of(t->rank, t->depth, id);
            if (oracle_unit_hash(seed ^ 0x5bd1e995ull, pass, parent) < pc && level > min_level)
                s = ST_COARSEN;
        }
        out[p] = s;
    }
}

/* ------------------------------------------------------------ init */
/* amr_solver::initialize, amr_solver.hpp:105-145, with cell centres from
 * physics_system::cell_coord (physics_system.hpp:107-138), plus noise. */
void oracle_init_state(oracle_tree* t, const double* bumps, int nbumps, double noise, uint64_t seed)
{
    const int    rank = t->rank, n = t->n, h = t->h;
    const size_t P1 = t->pad1;
    const double maxc = (double)(1u << t->depth);
    for (size_t p = 0; p < t->size; ++p) {
        uint32_t mc[3];
        int      level;
        oracle_decode(rank, t->ids[p], mc, &level);
        double cs[3], origin[3];
        cell_sizes(t, t->ids[p], cs);
        for (int k = 0; k < rank; ++k) origin[k] = 1.0 * (double)mc[k] / maxc;
        double*  u    = t->cur + p * t->pstride;
        uint64_t cell = 0;
        int      idx[3];
        for (idx[0] = h; idx[0] < n + h; ++idx[0])
            for (idx[1] = h; idx[1] < n + h; ++idx[1])
                for (idx[2] = (rank == 3 ? h : 0); idx[2] < (rank == 3 ? n + h : 1); ++idx[2]) {
                    size_t li = 0;
                    for (int k = 0; k < rank; ++k) li = li * P1 + (size_t)idx[k];
                    double x[3];
                    for (int k = 0; k < rank; ++k) {
                        const double data_cell = (double)idx[rank - 1 - k] - (double)h;
                        const double co        = origin[k] + data_cell * cs[k];
                        x[k]                   = co + 0.5 * cs[k];
                    }
                    double val = 0.0;
                    for (int b = 0; b < nbumps; ++b) {
                        const double* bp = bumps + b * (rank + 2);
                        double        r2 = 0.0;
                        for (int k = 0; k < rank; ++k) {
                            const double diff = x[k] - bp[k];
                            r2 += diff * diff;
                        }
                        const double s = bp[rank], a = bp[rank + 1];
                        val += a * exp(-r2 / (2.0 * s * s));
                    }
                    u[li] = val;
                    if (noise != 0.0) u[li] += noise * (2.0 * oracle_unit_hash(seed, t->ids[p], cell) - 1.0);
                    ++cell;
                }
    }
}

void oracle_random_state(oracle_tree* t, uint64_t seed)
{
    for (size_t p = 0; p < t->size; ++p)
        for (size_t c = 0; c < t->pstride; ++c)
            t->cur[p * t->pstride + c] = oracle_unit_hash(seed, t->ids[p], c) - 0.5;
}
