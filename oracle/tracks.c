/* CPU restatement of skylens-stream-rs's track builder with
 * ConflictPolicy::Drop (crates/core/src/tracks.rs:190-259, 472-500,
 * 786-799): verified matches become graph edges between (image, feature)
 * nodes, the connected components become tracks unless two of their nodes
 * share an image or they are shorter than min_length, and select_tracks caps
 * their number.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU track builder and the timed
 * CPU baseline, never the product path. Integer work: pinned by the
 * reference's known-answer tests (conflicting_component_is_dropped,
 * short_and_invalid_matches_are_excluded, cap_prefers_long_then_wide_tracks,
 * order_independent; tests/test_oracle_tracks.py).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* One pair's verified matches: matches[first .. first + count) of a flat
 * (feature a, feature b) array (PairMatches, tracks.rs:44-50). */
typedef struct {
    uint32_t image_a, image_b;
    uint64_t first, count;
} orc_pair_matches;

typedef struct {
    uint64_t edges, invalid_matches, conflicts, too_short, truncated, tracks;
} orc_track_stats;

static int cmp_u64(const void *a, const void *b) {
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/* UnionFind (tracks.rs:160-186): find with path compression, link makes the
 * smaller representative the root. */
static uint64_t uf_find(uint64_t *parent, uint64_t x) {
    uint64_t r = x;
    while (parent[r] != r) r = parent[r];
    while (parent[x] != r) {
        const uint64_t nx = parent[x];
        parent[x] = r;
        x = nx;
    }
    return r;
}

typedef struct {
    uint64_t first;  /* first node (= root: the smallest node) */
    uint64_t start, len, span;
} orc_track_ref;

static int cmp_track_cap(const void *a, const void *b) {
    const orc_track_ref *x = (const orc_track_ref *)a, *y = (const orc_track_ref *)b;
    if (x->len != y->len) return x->len > y->len ? -1 : 1;    /* length descending */
    if (x->span != y->span) return x->span > y->span ? -1 : 1; /* image span descending */
    return x->first < y->first ? -1 : x->first > y->first;    /* first observation ascending */
}

static int cmp_track_first(const void *a, const void *b) {
    const orc_track_ref *x = (const orc_track_ref *)a, *y = (const orc_track_ref *)b;
    return x->first < y->first ? -1 : x->first > y->first;
}

/* build_tracks with ConflictPolicy::Drop (tracks.rs:190-259, 472-500) and
 * select_tracks (:786-799). nf[i]: features of image i. Tracks come out as
 * node lists (node = offset of its image + feature, so node order is (image,
 * feature) order): track t is nodes[toff[t] .. toff[t+1]). Returns the track
 * count; writes at most cap_tracks tracks / cap_nodes nodes. */
int64_t orc_build_tracks_drop(const uint32_t *nf, int64_t n_images, const orc_pair_matches *pairs, int64_t n_pairs,
                              const uint32_t *matches, int64_t min_length, int64_t max_tracks, uint64_t *toff,
                              int64_t cap_tracks, uint64_t *nodes_out, int64_t cap_nodes, orc_track_stats *st) {
    memset(st, 0, sizeof *st);
    uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n_images + 1));
    off[0] = 0;
    for (int64_t i = 0; i < n_images; ++i) off[i + 1] = off[i] + nf[i];
    const uint64_t n = off[n_images];
    uint32_t *node_image = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n + 1));
    for (int64_t i = 0; i < n_images; ++i)
        for (uint64_t x = off[i]; x < off[i + 1]; ++x) node_image[x] = (uint32_t)i;
    uint64_t total = 0;
    for (int64_t p = 0; p < n_pairs; ++p) total += pairs[p].count;
    uint64_t *edges = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(total + 1));
    uint64_t ne = 0;
    for (int64_t p = 0; p < n_pairs; ++p) {
        const orc_pair_matches *pm = &pairs[p];
        for (uint64_t k = 0; k < pm->count; ++k) {
            const uint32_t fa = matches[2 * (pm->first + k)], fb = matches[2 * (pm->first + k) + 1];
            const int ok = pm->image_a != pm->image_b && (int64_t)pm->image_a < n_images &&
                           (int64_t)pm->image_b < n_images && fa < nf[pm->image_a] && fb < nf[pm->image_b];
            if (!ok) {
                st->invalid_matches++;
                continue;
            }
            /* the smaller image first (flip), then (small node, large node) */
            const int flip = pm->image_a > pm->image_b;
            const uint32_t lo = flip ? pm->image_b : pm->image_a, hi = flip ? pm->image_a : pm->image_b;
            const uint32_t f_lo = flip ? fb : fa, f_hi = flip ? fa : fb;
            const uint64_t u = off[lo] + f_lo, v = off[hi] + f_hi;
            edges[ne++] = ((u < v ? u : v) << 32) | (u < v ? v : u);
        }
    }
    /* per-pair sort + dedup, then the global sort + dedup, leave the same set */
    qsort(edges, (size_t)ne, sizeof(uint64_t), cmp_u64);
    uint64_t nu = 0;
    for (uint64_t e = 0; e < ne; ++e)
        if (nu == 0 || edges[e] != edges[nu - 1]) edges[nu++] = edges[e];
    st->edges = nu;
    uint64_t *parent = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n + 1));
    for (uint64_t x = 0; x < n; ++x) parent[x] = x;
    for (uint64_t e = 0; e < nu; ++e) {
        const uint64_t ru = uf_find(parent, edges[e] >> 32), rv = uf_find(parent, edges[e] & 0xffffffffu);
        if (ru != rv) parent[ru > rv ? ru : rv] = ru < rv ? ru : rv;
    }
    /* members: the endpoints of the edges, grouped by representative, each
     * group in node order */
    uint8_t *used = (uint8_t *)calloc((size_t)(n + 1), 1);
    for (uint64_t e = 0; e < nu; ++e) used[edges[e] >> 32] = used[edges[e] & 0xffffffffu] = 1;
    uint64_t *key = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n + 1)); /* root << 32 | node */
    uint64_t nk = 0;
    for (uint64_t x = 0; x < n; ++x)
        if (used[x]) key[nk++] = (uf_find(parent, x) << 32) | x;
    qsort(key, (size_t)nk, sizeof(uint64_t), cmp_u64);
    orc_track_ref *tr = (orc_track_ref *)malloc(sizeof(orc_track_ref) * (size_t)(nk + 1));
    uint64_t *tnodes = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nk + 1));
    uint64_t ntr = 0, nn = 0;
    const int64_t min_len = min_length < 2 ? 2 : min_length;
    for (uint64_t a = 0; a < nk;) {
        uint64_t b = a;
        while (b < nk && (key[b] >> 32) == (key[a] >> 32)) ++b;
        int conflict = 0;
        for (uint64_t q = a + 1; q < b; ++q)
            if (node_image[key[q] & 0xffffffffu] == node_image[key[q - 1] & 0xffffffffu]) conflict = 1;
        if (conflict) {
            st->conflicts++;
        } else if ((int64_t)(b - a) < min_len) {
            st->too_short++;
        } else {
            tr[ntr].first = key[a] & 0xffffffffu;
            tr[ntr].start = nn;
            tr[ntr].len = b - a;
            tr[ntr].span = node_image[key[b - 1] & 0xffffffffu] - node_image[key[a] & 0xffffffffu];
            for (uint64_t q = a; q < b; ++q) tnodes[nn++] = key[q] & 0xffffffffu;
            ++ntr;
        }
        a = b;
    }
    /* select_tracks: keep the longest, then widest, then first-observed */
    uint64_t keep = ntr;
    if ((int64_t)ntr > max_tracks) {
        qsort(tr, (size_t)ntr, sizeof(orc_track_ref), cmp_track_cap);
        keep = (uint64_t)max_tracks;
    }
    st->truncated = ntr - keep;
    qsort(tr, (size_t)keep, sizeof(orc_track_ref), cmp_track_first);
    st->tracks = keep;
    uint64_t w = 0;
    if (toff && cap_tracks > 0) toff[0] = 0;
    for (uint64_t t = 0; t < keep; ++t) {
        for (uint64_t q = 0; q < tr[t].len; ++q, ++w)
            if ((int64_t)w < cap_nodes && nodes_out) nodes_out[w] = tnodes[tr[t].start + q];
        if (toff && (int64_t)(t + 1) <= cap_tracks) toff[t + 1] = w;
    }
    free(off);
    free(node_image);
    free(edges);
    free(parent);
    free(used);
    free(key);
    free(tr);
    free(tnodes);
    return (int64_t)keep;
}
