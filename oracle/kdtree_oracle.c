/*
 * kdtree_oracle.c -- exact k nearest photons on the CPU through a kd-tree:
 * the gather of the benchmark's CPU baseline and reference arm.
 * TEST INFRASTRUCTURE ONLY.
 *
 * Build: median splits along the longest axis of each node's bounding box
 * (quickselect), down to leaves of at most PMO_KD_LEAF records, nodes
 * holding their tight boxes; the top levels in parallel (OpenMP tasks).
 * Query: depth-first, nearer child first, a node skipped only when its box
 * is strictly farther than the current k-th key's distance or than the
 * radius cap. The box distance takes the same rounded operations as a point
 * distance (|lo - q| <= |p - q| per axis for any p in the box, rounding is
 * monotone), so it never exceeds a contained point's distance and the result
 * is exactly the brute-force set under the key (float bits of d^2, photon
 * index) -- the same sets pmo_grid_knn and the GPU find.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "physical_oracle.h"

#define PMO_KD_LEAF 16
#define PMO_KD_STACK 128

typedef struct {
    float lo[3], hi[3];
    uint32_t begin, end;  /* records idx[begin, end) */
    int32_t left, right;  /* children, -1 for a leaf */
} kd_node;

struct pmo_kd {
    const float (*pos)[4];
    uint32_t n;
    uint32_t *idx;
    kd_node *nodes;
    uint32_t nnodes;
};

static uint32_t f2u_kd(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float u2f_kd(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* Nodes of a tree over n records: a node of more than PMO_KD_LEAF records
 * has two children of floor and ceil halves. */
static uint32_t count_nodes(uint32_t n) {
    if (n <= PMO_KD_LEAF) return 1;
    return 1 + count_nodes(n / 2) + count_nodes(n - n / 2);
}

/* Reorders idx[0, n) so that idx[m] holds the record of rank m along axis
 * a (ties by index), smaller ones before it, larger after (Hoare
 * quickselect with a median-of-three pivot). */
static int kd_less(const float (*pos)[4], int a, uint32_t i, uint32_t j) {
    float x = pos[i][a], y = pos[j][a];
    return x < y || (x == y && i < j);
}

static void kd_select(const float (*pos)[4], int a, uint32_t *idx, uint32_t n, uint32_t m) {
    uint32_t lo = 0, hi = n - 1;
    while (hi > lo) {
        uint32_t mid = lo + (hi - lo) / 2;
        /* median of three to idx[mid] */
        if (kd_less(pos, a, idx[mid], idx[lo])) { uint32_t t = idx[mid]; idx[mid] = idx[lo]; idx[lo] = t; }
        if (kd_less(pos, a, idx[hi], idx[lo])) { uint32_t t = idx[hi]; idx[hi] = idx[lo]; idx[lo] = t; }
        if (kd_less(pos, a, idx[hi], idx[mid])) { uint32_t t = idx[hi]; idx[hi] = idx[mid]; idx[mid] = t; }
        const uint32_t pv = idx[mid];
        uint32_t i = lo, j = hi;
        while (i <= j) {
            while (kd_less(pos, a, idx[i], pv)) ++i;
            while (kd_less(pos, a, pv, idx[j])) --j;
            if (i <= j) {
                uint32_t t = idx[i]; idx[i] = idx[j]; idx[j] = t;
                ++i;
                if (j == 0) break;
                --j;
            }
        }
        if (m <= j) hi = j;
        else if (m >= i) lo = i;
        else return;
    }
}

static void kd_build_node(struct pmo_kd *t, uint32_t node, uint32_t begin, uint32_t end, int depth) {
    kd_node *nd = &t->nodes[node];
    nd->begin = begin;
    nd->end = end;
    for (int a = 0; a < 3; ++a) { nd->lo[a] = INFINITY; nd->hi[a] = -INFINITY; }
    for (uint32_t i = begin; i < end; ++i) {
        const float *p = t->pos[t->idx[i]];
        for (int a = 0; a < 3; ++a) {
            if (p[a] < nd->lo[a]) nd->lo[a] = p[a];
            if (p[a] > nd->hi[a]) nd->hi[a] = p[a];
        }
    }
    const uint32_t n = end - begin;
    if (n <= PMO_KD_LEAF) {
        nd->left = nd->right = -1;
        return;
    }
    int axis = 0;
    float ext = nd->hi[0] - nd->lo[0];
    for (int a = 1; a < 3; ++a)
        if (nd->hi[a] - nd->lo[a] > ext) { ext = nd->hi[a] - nd->lo[a]; axis = a; }
    const uint32_t half = n / 2;
    kd_select(t->pos, axis, t->idx + begin, n, half);
    const uint32_t left = node + 1;
    const uint32_t right = left + count_nodes(half);
    nd->left = (int32_t)left;
    nd->right = (int32_t)right;
    if (depth < 6) {
#pragma omp task
        kd_build_node(t, left, begin, begin + half, depth + 1);
#pragma omp task
        kd_build_node(t, right, begin + half, end, depth + 1);
#pragma omp taskwait
    } else {
        kd_build_node(t, left, begin, begin + half, depth + 1);
        kd_build_node(t, right, begin + half, end, depth + 1);
    }
}

pmo_kd *pmo_kd_build(const float (*pos)[4], uint32_t n) {
    pmo_kd *t = calloc(1, sizeof(pmo_kd));
    if (!t) return NULL;
    t->pos = pos;
    t->n = n;
    t->idx = malloc(sizeof(uint32_t) * (n ? n : 1));
    t->nnodes = n ? count_nodes(n) : 0;
    t->nodes = malloc(sizeof(kd_node) * (t->nnodes ? t->nnodes : 1));
    if (!t->idx || !t->nodes) {
        pmo_kd_free(t);
        return NULL;
    }
    for (uint32_t i = 0; i < n; ++i) t->idx[i] = i;
    if (n) {
#pragma omp parallel
#pragma omp single
        kd_build_node(t, 0, 0, n, 0);
    }
    return t;
}

void pmo_kd_free(pmo_kd *t) {
    if (!t) return;
    free(t->idx);
    free(t->nodes);
    free(t);
}

static float box_d2(const kd_node *nd, const float q[3]) {
    float d[3];
    for (int a = 0; a < 3; ++a) {
        float v = 0.0f;
        if (q[a] < nd->lo[a]) v = nd->lo[a] - q[a];
        else if (q[a] > nd->hi[a]) v = q[a] - nd->hi[a];
        d[a] = v;
    }
    return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}

/* The k smallest keys (float bits of d^2 << 32 | photon index from pos[3])
 * with d^2 <= r2, ascending; returns the count (pmo_grid_knn's contract). */
int pmo_kd_knn(const pmo_kd *t, const float q[3], int k, float r2, uint64_t *keys) {
    int cnt = 0;
    if (!t || t->n == 0 || k <= 0) return 0;
    uint32_t stack[PMO_KD_STACK];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const kd_node *nd = &t->nodes[stack[--sp]];
        const float bd = box_d2(nd, q);
        if (bd > r2) continue;
        if (cnt == k && bd > u2f_kd((uint32_t)(keys[k - 1] >> 32))) continue;
        if (nd->left < 0) {
            for (uint32_t it = nd->begin; it < nd->end; ++it) {
                const float *p = t->pos[t->idx[it]];
                float dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
                float d2 = dx * dx + dy * dy + dz * dz;
                if (!(d2 <= r2)) continue;
                uint64_t key = ((uint64_t)f2u_kd(d2) << 32) | f2u_kd(p[3]);
                if (cnt == k && key >= keys[k - 1]) continue;
                int j = cnt < k ? cnt++ : k - 1;
                while (j > 0 && keys[j - 1] > key) { keys[j] = keys[j - 1]; --j; }
                keys[j] = key;
            }
            continue;
        }
        /* nearer child on top of the stack */
        const kd_node *l = &t->nodes[nd->left], *r = &t->nodes[nd->right];
        const float dl = box_d2(l, q), dr = box_d2(r, q);
        if (sp + 2 > PMO_KD_STACK) continue;  /* depth is log2(n / 16) + 1 < 64 */
        if (dl <= dr) {
            stack[sp++] = (uint32_t)nd->right;
            stack[sp++] = (uint32_t)nd->left;
        } else {
            stack[sp++] = (uint32_t)nd->left;
            stack[sp++] = (uint32_t)nd->right;
        }
    }
    return cnt;
}

void pmo_knn_kd(const float (*pos)[4], uint32_t n, const float (*queries)[4], uint32_t nq, int k,
                float radius, uint32_t *idx_out, float *d2_out) {
    float r2 = radius * radius;
    pmo_kd *t = pmo_kd_build(pos, n);
#pragma omp parallel for schedule(dynamic, 64)
    for (long qi = 0; qi < (long)nq; ++qi) {
        uint64_t keys[128];
        int c = pmo_kd_knn(t, queries[qi], k, r2, keys);
        for (int j = 0; j < k; ++j) {
            idx_out[qi * k + j] = j < c ? (uint32_t)keys[j] : 0xffffffffu;
            d2_out[qi * k + j] = j < c ? u2f_kd((uint32_t)(keys[j] >> 32)) : r2;
        }
    }
    pmo_kd_free(t);
}
