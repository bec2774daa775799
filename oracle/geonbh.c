/*
 * Oracle (test infrastructure, not product code): CPU restatement of the
 * geodesic-neighbourhood search of the reference's tangent-frame routine.
 *
 * Follows RVGP/lib/ptu_dijkstra.pyx:361-394 (per-point Dijkstra that stops once
 * K+1 nodes are scanned) and the Fibonacci-heap operations it uses,
 * ptu_dijkstra.pyx:444-690 (insert_node, decrease_val, link, remove_min and the
 * sibling helpers).  The heap is restated with index-linked arrays instead of
 * pointers and a per-source stamp replaces the reference's O(N) re-initialisation
 * of every node (pyx:364-365); the order of every heap operation is the same, so
 * ties between equal path lengths are broken exactly as the reference breaks them.
 *
 * Only tests, bench.py's CPU-baseline leg and __graft_entry__.smoke() call this.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NIL (-1)
enum { ST_SCANNED = 0, ST_NOT_IN_HEAP = 1, ST_IN_HEAP = 2 };

typedef struct {
    int n;
    double *val;
    int *rank, *parent, *left, *right, *child, *stamp;
    signed char *state;
    int min_node;
    int roots_by_rank[100];
} heap_t;

static int rightmost(heap_t *h, int v) { while (h->right[v] != NIL) v = h->right[v]; return v; }
static int leftmost(heap_t *h, int v) { while (h->left[v] != NIL) v = h->left[v]; return v; }

static void add_sibling(heap_t *h, int node, int s) {
    int t = rightmost(h, node);
    h->right[t] = s;
    h->left[s] = t;
    h->right[s] = NIL;
    h->parent[s] = h->parent[node];
    if (h->parent[s] != NIL) h->rank[h->parent[s]] += 1;
}

static void add_child(heap_t *h, int node, int c) {
    h->parent[c] = node;
    if (h->child[node] != NIL) {
        add_sibling(h, h->child[node], c);
    } else {
        h->child[node] = c;
        h->right[c] = NIL;
        h->left[c] = NIL;
        h->rank[node] = 1;
    }
}

static void unlink_node(heap_t *h, int v) {
    int p = h->parent[v];
    if (p != NIL) {
        h->rank[p] -= 1;
        if (h->left[v] != NIL) h->child[p] = h->left[v];
        else if (h->right[v] != NIL) h->child[p] = h->right[v];
        else h->child[p] = NIL;
    }
    if (h->left[v] != NIL) h->right[h->left[v]] = h->right[v];
    if (h->right[v] != NIL) h->left[h->right[v]] = h->left[v];
    h->left[v] = NIL;
    h->right[v] = NIL;
    h->parent[v] = NIL;
}

static void insert_node(heap_t *h, int v) {
    if (h->min_node != NIL) {
        add_sibling(h, h->min_node, v);
        if (h->val[v] < h->val[h->min_node]) h->min_node = v;
    } else {
        h->min_node = v;
    }
}

static void decrease_val(heap_t *h, int v, double newval) {
    h->val[v] = newval;
    if (h->parent[v] != NIL && h->val[h->parent[v]] >= newval) {
        unlink_node(h, v);
        insert_node(h, v);
    } else if (h->val[h->min_node] > h->val[v]) {
        h->min_node = v;
    }
}

static void link_root(heap_t *h, int v) {
    for (;;) {
        int r = h->rank[v];
        int other = h->roots_by_rank[r];
        if (other == NIL) { h->roots_by_rank[r] = v; return; }
        h->roots_by_rank[r] = NIL;
        if (h->val[v] < h->val[other] || v == h->min_node) {
            unlink_node(h, other);
            add_child(h, v, other);
        } else {
            unlink_node(h, v);
            add_child(h, other, v);
            v = other;
        }
    }
}

static int remove_min(heap_t *h) {
    int m = h->min_node, t, tr, out;
    if (h->child[m] != NIL) {
        t = leftmost(h, h->child[m]);
        while (t != NIL) {
            tr = h->right[t];
            unlink_node(h, t);
            add_sibling(h, m, t);
            t = tr;
        }
        h->child[m] = NIL;
    }
    t = leftmost(h, m);
    if (t == m) {
        if (h->right[m] != NIL) {
            t = h->right[m];
        } else {
            out = m;
            h->min_node = NIL;
            return out;
        }
    }
    out = m;
    unlink_node(h, m);
    h->min_node = t;
    for (int i = 0; i < 100; ++i) h->roots_by_rank[i] = NIL;
    while (t != NIL) {
        if (h->val[t] < h->val[h->min_node]) h->min_node = t;
        tr = h->right[t];
        link_root(h, t);
        t = tr;
    }
    return out;
}

static void touch(heap_t *h, int v, int src) {
    if (h->stamp[v] != src) {
        h->stamp[v] = src;
        h->val[v] = 0.0;
        h->rank[v] = 0;
        h->state[v] = ST_NOT_IN_HEAP;
        h->parent[v] = h->left[v] = h->right[v] = h->child[v] = NIL;
    }
}

/*
 * For every source i in [0, n): the first K+1 nodes popped by the heap-based
 * Dijkstra over CSR (indptr, indices, weights) are written to out[i*(K+1) ...],
 * in pop order.  Returns 0, or the 1-based index of the first source whose
 * component holds fewer than K+1 nodes (its row is then padded with -1).
 */
int oracle_geodesic_neighbourhoods(int n, const int *indptr, const int *indices,
                                   const double *weights, int K, int *out) {
    heap_t h;
    int status = 0;
    h.n = n;
    h.val = (double *)malloc(sizeof(double) * (size_t)n);
    h.rank = (int *)malloc(sizeof(int) * (size_t)n);
    h.parent = (int *)malloc(sizeof(int) * (size_t)n);
    h.left = (int *)malloc(sizeof(int) * (size_t)n);
    h.right = (int *)malloc(sizeof(int) * (size_t)n);
    h.child = (int *)malloc(sizeof(int) * (size_t)n);
    h.stamp = (int *)malloc(sizeof(int) * (size_t)n);
    h.state = (signed char *)malloc((size_t)n);
    for (int v = 0; v < n; ++v) h.stamp[v] = -1;
    for (int i = 0; i < 100; ++i) h.roots_by_rank[i] = NIL;

    for (int i = 0; i < n; ++i) {
        int *row = out + (size_t)i * (size_t)(K + 1);
        int scanned = 0;
        touch(&h, i, i);
        h.min_node = NIL;
        insert_node(&h, i);
        while (h.min_node != NIL && scanned <= K) {
            int v = remove_min(&h);
            h.state[v] = ST_SCANNED;
            row[scanned++] = v;
            if (scanned <= K) {
                for (int e = indptr[v]; e < indptr[v + 1]; ++e) {
                    int u = indices[e];
                    touch(&h, u, i);
                    if (h.state[u] != ST_SCANNED) {
                        double nv = h.val[v] + weights[e];
                        if (h.state[u] == ST_NOT_IN_HEAP) {
                            h.state[u] = ST_IN_HEAP;
                            h.val[u] = nv;
                            insert_node(&h, u);
                        } else if (h.val[u] > nv) {
                            decrease_val(&h, u, nv);
                        }
                    }
                }
            }
        }
        if (scanned < K + 1) {
            for (int q = scanned; q <= K; ++q) row[q] = -1;
            if (!status) status = i + 1;
        }
    }
    free(h.val); free(h.rank); free(h.parent); free(h.left); free(h.right);
    free(h.child); free(h.stamp); free(h.state);
    return status;
}
