// Mesh connectivity on the device: the reference's compute_mesh_edges, compute_patches and
// compute_chains (src/mesh_connectivity.cpp:10-56, 58-92 / 152-186, 190-242) over a finished mesh.
//
// Edges.  Every face corner j of face f is an occurrence of the edge (v_j, v_{j+1}) at position
// face_offsets[f] + j, which is the reference's visiting order.  Occurrences lower their key's owner
// to their position with atomicMin; an occurrence is new iff it owns its key; a scan numbers the new
// ones.  That is the reference's first-occurrence numbering.  Each edge lists its occurrences as
// (face, local edge), in occurrence order.
//
// Patches and chains are breadth-first searches from the smallest unvisited node, in node order,
// over a graph whose node order and slot order fix the result:
//   patches: nodes are faces, the slots of a face are its edges in order, and a slot leads to the
//            other face of a manifold edge (exactly two occurrences);
//   chains:  nodes are the non-manifold edges (more than two occurrences) in edge order, the slots
//            of an edge are its two end vertices, and a slot leads to the other non-manifold edge of
//            a vertex that has exactly two.
// Here:
//   1. connected components by union-find with the larger root hooked under the smaller, so every
//      root is its component's smallest node, and the components come in the reference's order;
//   2. one breadth-first search per level over all components at once: a node of the next level
//      belongs to the frontier slot that reaches it first in the reference's queue order, which is
//      the smallest (frontier position, slot) key (atomicMin); the next frontier is written in key
//      order (a scan of the per-node counts);
//   3. a stable sort of the discovery sequence by component gives every component's node list in
//      its queue order.
#include "extract_common.cuh"
#include "launch.hpp"

namespace ria {

using namespace xc;

namespace {

constexpr int kMaxUnionSteps = 1 << 20;

__global__ void k_iota_u32(int64_t n, uint32_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) out[i] = (uint32_t)i;
}

// offsets of two slots per node: out[i] = 2 i
__global__ void k_iota2_i64(int64_t n, int64_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) out[i] = 2 * i;
}

__global__ void k_histogram(int64_t n, const uint32_t* __restrict__ key, uint32_t* __restrict__ count) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) atomicAdd(&count[key[i]], 1u);
}

__global__ void k_set_total(int64_t* __restrict__ off, int64_t n, int64_t total) { off[n] = total; }

// ---- edges

__global__ void k_edge_keys(int64_t n_faces, const int64_t* __restrict__ fo, const int64_t* __restrict__ fv,
                            HashTab64 h, uint32_t* __restrict__ occ_slot, uint32_t* __restrict__ occ_face,
                            uint32_t* status) {
    const int64_t f = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (f >= n_faces) return;
    const int64_t b = fo[f], L = fo[f + 1] - b;
    for (int64_t j = 0; j < L; ++j) {
        int64_t v1 = fv[b + j], v2 = fv[b + (j + 1 == L ? 0 : j + 1)];
        if (v1 > v2) {
            const int64_t t = v1;
            v1 = v2;
            v2 = t;
        }
        const int64_t s = ht64_insert_min(h, ((uint64_t)v1 << 32) | (uint64_t)v2, (uint32_t)(b + j));
        if (s < 0) raise_status(status, ST_HASH_FULL);
        occ_slot[b + j] = (uint32_t)(s < 0 ? 0 : s);
        occ_face[b + j] = (uint32_t)f;
    }
}

__global__ void k_edge_owner(int64_t n, const HashTab64 h, const uint32_t* __restrict__ occ_slot,
                             uint32_t* __restrict__ own, uint32_t* __restrict__ flag, uint32_t* __restrict__ cnt) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint32_t o = h.owner[occ_slot[p]];
    own[p] = o;
    flag[p] = o == (uint32_t)p;
    atomicAdd(&cnt[o], 1u);
}

// edge of every occurrence, the new edges' end vertices and occurrence counts
__global__ void k_edge_emit(int64_t n, const int64_t* __restrict__ fo, const int64_t* __restrict__ fv,
                            const uint32_t* __restrict__ occ_face, const uint32_t* __restrict__ own,
                            const uint32_t* __restrict__ eid, const uint32_t* __restrict__ cnt,
                            int64_t* __restrict__ face_edges, int64_t* __restrict__ edges,
                            uint32_t* __restrict__ edge_cnt) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint32_t o = own[p];
    const uint32_t e = eid[o];
    face_edges[p] = e;
    if (o != (uint32_t)p) return;
    const int64_t f = occ_face[p], b = fo[f], L = fo[f + 1] - b, j = p - b;
    int64_t v1 = fv[p], v2 = fv[b + (j + 1 == L ? 0 : j + 1)];
    if (v1 > v2) {
        const int64_t t = v1;
        v1 = v2;
        v2 = t;
    }
    edges[2 * (int64_t)e] = v1;
    edges[2 * (int64_t)e + 1] = v2;
    edge_cnt[e] = cnt[p];
}

__global__ void k_edge_fill(int64_t n, const int64_t* __restrict__ face_edges, const uint32_t* __restrict__ eoff,
                            uint32_t* __restrict__ fill, uint32_t* __restrict__ occ) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const int64_t e = face_edges[p];
    occ[eoff[e] + atomicAdd(&fill[e], 1u)] = (uint32_t)p;
}

// each edge's occurrences in position order, as (face, local edge)
__global__ void k_edge_sort(int64_t n_edges, const uint32_t* __restrict__ eoff, const uint32_t* __restrict__ edge_cnt,
                            uint32_t* __restrict__ occ, const uint32_t* __restrict__ occ_face,
                            const int64_t* __restrict__ fo, int64_t* __restrict__ edge_faces,
                            int64_t* __restrict__ edge_face_offsets) {
    const int64_t e = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (e >= n_edges) return;
    const uint32_t b = eoff[e], c = edge_cnt[e];
    uint32_t* o = occ + b;
    for (uint32_t x = 1; x < c; ++x)
        for (uint32_t y = x; y > 0 && o[y - 1] > o[y]; --y) {
            const uint32_t t = o[y];
            o[y] = o[y - 1];
            o[y - 1] = t;
        }
    edge_face_offsets[e] = b;
    for (uint32_t x = 0; x < c; ++x) {
        const int64_t f = occ_face[o[x]];
        edge_faces[2 * ((int64_t)b + x)] = f;
        edge_faces[2 * ((int64_t)b + x) + 1] = (int64_t)o[x] - fo[f];
    }
}

// ---- graphs for the searches: adj[adj_off[u] .. adj_off[u + 1]) = node reached by each slot, or -1

__global__ void k_patch_adj(int64_t n, const int64_t* __restrict__ face_edges, const uint32_t* __restrict__ occ_face,
                            const uint32_t* __restrict__ eoff, const uint32_t* __restrict__ edge_cnt,
                            const uint32_t* __restrict__ occ, int32_t* __restrict__ adj) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const int64_t e = face_edges[p];
    int32_t nb = -1;
    if (edge_cnt[e] == 2) {  // manifold edge: the other face (src/mesh_connectivity.cpp:80-84)
        const uint32_t f = occ_face[p], f0 = occ_face[occ[eoff[e]]], f1 = occ_face[occ[eoff[e] + 1]];
        nb = (int32_t)(f0 == f ? f1 : f0);
    }
    adj[p] = nb;
}

// non-manifold edges: their local index (in edge order) and per vertex the count and first two
__global__ void k_nm_mark(int64_t n_edges, const uint32_t* __restrict__ edge_cnt, uint32_t* __restrict__ nm_flag) {
    const int64_t e = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (e < n_edges) nm_flag[e] = edge_cnt[e] > 2;
}

__global__ void k_nm_vert(int64_t n_edges, const uint32_t* __restrict__ nm_flag, const uint32_t* __restrict__ nm_id,
                          const int64_t* __restrict__ edges, uint32_t* __restrict__ vcnt, int32_t* __restrict__ vedge) {
    const int64_t e = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (e >= n_edges || !nm_flag[e]) return;
    for (int s = 0; s < 2; ++s) {
        const int64_t v = edges[2 * e + s];
        const uint32_t k = atomicAdd(&vcnt[v], 1u);
        if (k < 2) vedge[2 * v + k] = (int32_t)nm_id[e];
    }
}

__global__ void k_chain_adj(int64_t n_edges, const uint32_t* __restrict__ nm_flag, const uint32_t* __restrict__ nm_id,
                            const int64_t* __restrict__ edges, const uint32_t* __restrict__ vcnt,
                            const int32_t* __restrict__ vedge, int32_t* __restrict__ adj, int64_t* __restrict__ nm_edge) {
    const int64_t e = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (e >= n_edges || !nm_flag[e]) return;
    const uint32_t me = nm_id[e];
    nm_edge[me] = e;
    for (int s = 0; s < 2; ++s) {  // v1, then v2 (src/mesh_connectivity.cpp:210-238)
        const int64_t v = edges[2 * e + s];
        int32_t nb = -1;
        if (vcnt[v] == 2) nb = vedge[2 * v] == (int32_t)me ? vedge[2 * v + 1] : vedge[2 * v];
        adj[2 * (int64_t)me + s] = nb;
    }
}

// ---- components: union-find, the smaller root wins

// root of x, halving the path on the way: a node is re-pointed to its grandparent, which is also one
// of its ancestors (parents only ever point to smaller nodes, so there are no cycles)
__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x) {
    for (int i = 0; i < kMaxUnionSteps; ++i) {
        const uint32_t p = parent[x];
        if (p == x) return x;
        const uint32_t g = parent[p];
        if (g != p) parent[x] = g;
        x = g;
    }
    return x;
}

template <class Off>
__global__ void k_union(int64_t n, const Off* __restrict__ adj_off, const int32_t* __restrict__ adj,
                        uint32_t* __restrict__ parent, uint32_t* status) {
    const int64_t u = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (u >= n) return;
    for (int64_t s = adj_off[u]; s < adj_off[u + 1]; ++s) {
        const int32_t v = adj[s];
        if (v < 0 || v <= u) continue;  // each link once, from its smaller end
        uint32_t a = (uint32_t)u, b = (uint32_t)v;
        int step = 0;
        for (; step < kMaxUnionSteps; ++step) {
            a = uf_find(parent, a);
            b = uf_find(parent, b);
            if (a == b) break;
            if (a > b) {
                const uint32_t t = a;
                a = b;
                b = t;
            }
            // hook the larger root under the smaller one
            if (atomicCAS(&parent[b], b, a) == b) break;
        }
        if (step == kMaxUnionSteps) raise_status(status, ST_INTERNAL);
    }
}

// root of x without writing: after the unions only the thread of node x may write parent[x], so
// that every node ends pointing at its root (a halving write from another thread could replace the
// root with an intermediate ancestor)
__device__ __forceinline__ uint32_t uf_root(const uint32_t* parent, uint32_t x) {
    for (int i = 0; i < kMaxUnionSteps; ++i) {
        const uint32_t p = parent[x];
        if (p == x) return x;
        x = p;
    }
    return x;
}

__global__ void k_compress(int64_t n, uint32_t* __restrict__ parent, uint32_t* __restrict__ seed) {
    const int64_t u = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (u >= n) return;
    const uint32_t r = uf_root(parent, (uint32_t)u);
    parent[u] = r;
    seed[u] = r == (uint32_t)u;
}

// ---- ordered breadth-first search

__global__ void k_bfs_init(int64_t n, const uint32_t* __restrict__ seed, const uint32_t* __restrict__ comp_of_seed,
                           int32_t* __restrict__ frontier, uint8_t* __restrict__ visited,
                           unsigned long long* __restrict__ claim) {
    const int64_t u = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (u >= n) return;
    claim[u] = ~0ull;
    visited[u] = seed[u] ? 1 : 0;
    if (seed[u]) frontier[comp_of_seed[u]] = (int32_t)u;
}

template <class Off>
__global__ void k_bfs_claim(int64_t nf, const int32_t* __restrict__ frontier, const Off* __restrict__ adj_off,
                            const int32_t* __restrict__ adj, const uint8_t* __restrict__ visited,
                            unsigned long long* __restrict__ claim) {
    const int64_t k = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (k >= nf) return;
    const int32_t u = frontier[k];
    const int64_t b = adj_off[u];
    for (int64_t s = b; s < adj_off[u + 1]; ++s) {
        const int32_t v = adj[s];
        if (v >= 0 && !visited[v]) atomicMin(&claim[v], ((unsigned long long)k << 16) | (unsigned long long)(s - b));
    }
}

template <class Off>
__global__ void k_bfs_count(int64_t nf, const int32_t* __restrict__ frontier, const Off* __restrict__ adj_off,
                            const int32_t* __restrict__ adj, const uint8_t* __restrict__ visited,
                            const unsigned long long* __restrict__ claim, uint32_t* __restrict__ won) {
    const int64_t k = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (k >= nf) return;
    const int32_t u = frontier[k];
    const int64_t b = adj_off[u];
    uint32_t c = 0;
    for (int64_t s = b; s < adj_off[u + 1]; ++s) {
        const int32_t v = adj[s];
        if (v >= 0 && !visited[v] && claim[v] == (((unsigned long long)k << 16) | (unsigned long long)(s - b))) ++c;
    }
    won[k] = c;
}

// the next frontier in key order; it is also appended to the discovery sequence
template <class Off>
__global__ void k_bfs_next(int64_t nf, const int32_t* __restrict__ frontier, const Off* __restrict__ adj_off,
                           const int32_t* __restrict__ adj, uint8_t* __restrict__ visited,
                           const unsigned long long* __restrict__ claim, const uint32_t* __restrict__ woff,
                           int32_t* __restrict__ next, int32_t* __restrict__ disc) {
    const int64_t k = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (k >= nf) return;
    const int32_t u = frontier[k];
    const int64_t b = adj_off[u];
    uint32_t o = woff[k];
    for (int64_t s = b; s < adj_off[u + 1]; ++s) {
        const int32_t v = adj[s];
        if (v >= 0 && !visited[v] && claim[v] == (((unsigned long long)k << 16) | (unsigned long long)(s - b))) {
            next[o] = v;
            disc[o] = v;
            ++o;
        }
    }
}

__global__ void k_mark_visited(int64_t n, const int32_t* __restrict__ list, uint8_t* __restrict__ visited) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) visited[list[i]] = 1;
}

__global__ void k_comp_keys(int64_t n, const int32_t* __restrict__ disc, const uint32_t* __restrict__ parent,
                            const uint32_t* __restrict__ comp_of_seed, uint32_t* __restrict__ key) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) key[i] = comp_of_seed[parent[disc[i]]];
}

__global__ void k_to_i64(int64_t n, const int32_t* __restrict__ in, const int64_t* __restrict__ map,
                         int64_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) out[i] = map ? map[in[i]] : (int64_t)in[i];
}

__global__ void k_u32_to_i64(int64_t n, const uint32_t* __restrict__ in, int64_t* __restrict__ out, int64_t total) {
    const int64_t i = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (i < n) out[i] = in[i];
    if (i == n) out[n] = total;
}

__global__ void k_patch_labels(int64_t n_comp, const int64_t* __restrict__ comp_off, const int64_t* __restrict__ order,
                               const int64_t* __restrict__ face_func, int64_t* __restrict__ labels) {
    const int64_t c = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (c >= n_comp) return;
    const int64_t f = order[comp_off[c]];
    labels[2 * c] = face_func[2 * f];
    labels[2 * c + 1] = face_func[2 * f + 1];
}

// Components of a graph of n nodes and their nodes in breadth-first order from each component's
// smallest node.  Allocates comp_off [n_comp + 1] and order [n] (int64; `map` renames the nodes).
template <class Off>
cudaError_t ordered_bfs(int64_t n, const Off* adj_off, const int32_t* adj, const int64_t* map, int64_t** comp_off,
                        int64_t* n_comp, int64_t** order, uint32_t* status, Pool& pool, cudaStream_t s) {
    *n_comp = 0;
    cudaError_t e;
    if ((e = cudaMallocAsync((void**)order, sizeof(int64_t) * (size_t)(n > 0 ? n : 1), s)) != cudaSuccess) return e;
    if (n == 0) {
        if ((e = cudaMallocAsync((void**)comp_off, sizeof(int64_t), s)) != cudaSuccess) return e;
        return cudaMemsetAsync(*comp_off, 0, sizeof(int64_t), s);
    }
    uint32_t* parent = pool.get<uint32_t>(n);
    uint32_t* seed = pool.get<uint32_t>(n);
    uint32_t* cseed = pool.get<uint32_t>(n);
    int32_t* fa = pool.get<int32_t>(n);
    int32_t* fb = pool.get<int32_t>(n);
    int32_t* disc = pool.get<int32_t>(n);
    uint8_t* visited = pool.get<uint8_t>(n);
    unsigned long long* claim = pool.get<unsigned long long>(n);
    uint32_t* won = pool.get<uint32_t>(n);
    uint32_t* woff = pool.get<uint32_t>(n);
    if (pool.err) return pool.err;
    k_iota_u32<<<nblk(n), kBs, 0, s>>>(n, parent);
    note_launch();
    k_union<Off><<<nblk(n), kBs, 0, s>>>(n, adj_off, adj, parent, status);
    note_launch();
    k_compress<<<nblk(n), kBs, 0, s>>>(n, parent, seed);
    note_launch();
    if ((e = exscan_u32(seed, cseed, n, s)) != cudaSuccess) return e;
    if ((e = scan_total(seed, cseed, n, n_comp, s)) != cudaSuccess) return e;
    k_bfs_init<<<nblk(n), kBs, 0, s>>>(n, seed, cseed, fa, visited, claim);
    note_launch();
    // the seeds open the discovery sequence, in component order
    if ((e = cudaMemcpyAsync(disc, fa, sizeof(int32_t) * (size_t)*n_comp, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return e;
    int64_t nf = *n_comp, done = *n_comp;
    int32_t* cur = fa;
    int32_t* nxt = fb;
    while (nf > 0) {
        k_bfs_claim<Off><<<nblk(nf), kBs, 0, s>>>(nf, cur, adj_off, adj, visited, claim);
        note_launch();
        k_bfs_count<Off><<<nblk(nf), kBs, 0, s>>>(nf, cur, adj_off, adj, visited, claim, won);
        note_launch();
        if ((e = exscan_u32(won, woff, nf, s)) != cudaSuccess) return e;
        int64_t nn = 0;
        if ((e = scan_total(won, woff, nf, &nn, s)) != cudaSuccess) return e;
        if (done + nn > n) return cudaErrorUnknown;
        k_bfs_next<Off><<<nblk(nf), kBs, 0, s>>>(nf, cur, adj_off, adj, visited, claim, woff, nxt, disc + done);
        note_launch();
        if (nn > 0) {
            k_mark_visited<<<nblk(nn), kBs, 0, s>>>(nn, nxt, visited);
            note_launch();
        }
        done += nn;
        nf = nn;
        int32_t* t = cur;
        cur = nxt;
        nxt = t;
    }
    if (done != n) return cudaErrorUnknown;  // every node is reached from its component's root
    // stable sort of the discovery sequence by component
    uint32_t* key = pool.get<uint32_t>(n);
    uint32_t* key_sorted = pool.get<uint32_t>(n);
    int32_t* node_sorted = pool.get<int32_t>(n);
    uint32_t* csize = pool.get<uint32_t>(*n_comp);
    uint32_t* coff = pool.get<uint32_t>(*n_comp);
    if (pool.err) return pool.err;
    k_comp_keys<<<nblk(n), kBs, 0, s>>>(n, disc, parent, cseed, key);
    note_launch();
    int end_bit = 1;
    while (end_bit < 32 && (1ll << end_bit) < *n_comp) ++end_bit;
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, key, key_sorted, disc, node_sorted, (int)n, 0, end_bit, s);
    void* tmp = pool.get<uint8_t>((int64_t)bytes);
    if (pool.err) return pool.err;
    if ((e = cub::DeviceRadixSort::SortPairs(tmp, bytes, key, key_sorted, disc, node_sorted, (int)n, 0, end_bit, s)) !=
        cudaSuccess)
        return e;
    k_to_i64<<<nblk(n), kBs, 0, s>>>(n, node_sorted, map, *order);
    note_launch();
    // component offsets from the component sizes
    if ((e = cudaMemsetAsync(csize, 0, sizeof(uint32_t) * (size_t)*n_comp, s)) != cudaSuccess) return e;
    k_histogram<<<nblk(n), kBs, 0, s>>>(n, key_sorted, csize);
    note_launch();
    if ((e = exscan_u32(csize, coff, *n_comp, s)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync((void**)comp_off, sizeof(int64_t) * (size_t)(*n_comp + 1), s)) != cudaSuccess) return e;
    k_u32_to_i64<<<nblk(*n_comp + 1), kBs, 0, s>>>(*n_comp, coff, *comp_off, n);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t build_connectivity(const ConnArgs& a, ConnOut& out, cudaStream_t s) {
    Pool pool{s};
    out = ConnOut();
    const int64_t NF = a.n_faces, NO = a.n_face_verts;
    if (NO >= (1ll << 32) - 1 || NF >= (1ll << 31) - 1) return cudaErrorInvalidValue;
    cudaError_t e;
    uint32_t* status = pool.get<uint32_t>(1);
    const uint64_t cap = pow2_at_least(2 * (uint64_t)NO + 1);
    HashTab64 h{pool.get<unsigned long long>((int64_t)cap), pool.get<uint32_t>((int64_t)cap), cap - 1};
    uint32_t* occ_slot = pool.get<uint32_t>(NO);
    uint32_t* occ_face = pool.get<uint32_t>(NO);
    uint32_t* own = pool.get<uint32_t>(NO);
    uint32_t* flag = pool.get<uint32_t>(NO);
    uint32_t* cnt = pool.get<uint32_t>(NO);
    uint32_t* eid = pool.get<uint32_t>(NO);
    if (pool.err) return pool.err;
    cudaMemsetAsync(status, 0, 4, s);
    cudaMemsetAsync(h.keys, 0xFF, sizeof(unsigned long long) * cap, s);
    cudaMemsetAsync(h.owner, 0xFF, sizeof(uint32_t) * cap, s);
    cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)(NO > 0 ? NO : 1), s);
    if ((e = cudaMallocAsync((void**)&out.face_edges, sizeof(int64_t) * (size_t)(NO > 0 ? NO : 1), s)) != cudaSuccess)
        return e;
    if (NF > 0) {
        k_edge_keys<<<nblk(NF), kBs, 0, s>>>(NF, a.face_offsets, a.face_verts, h, occ_slot, occ_face, status);
        note_launch();
    }
    if (NO > 0) {
        k_edge_owner<<<nblk(NO), kBs, 0, s>>>(NO, h, occ_slot, own, flag, cnt);
        note_launch();
    }
    if ((e = exscan_u32(flag, eid, NO, s)) != cudaSuccess) return e;
    int64_t NE = 0;
    if ((e = scan_total(flag, eid, NO, &NE, s)) != cudaSuccess) return e;
    out.n_edges = NE;
    uint32_t* edge_cnt = pool.get<uint32_t>(NE);
    uint32_t* eoff = pool.get<uint32_t>(NE);
    uint32_t* fill = pool.get<uint32_t>(NE);
    uint32_t* occ = pool.get<uint32_t>(NO);
    if (pool.err) return pool.err;
    if ((e = cudaMallocAsync((void**)&out.edges, sizeof(int64_t) * 2 * (size_t)(NE > 0 ? NE : 1), s)) != cudaSuccess)
        return e;
    if ((e = cudaMallocAsync((void**)&out.edge_face_offsets, sizeof(int64_t) * (size_t)(NE + 1), s)) != cudaSuccess)
        return e;
    if ((e = cudaMallocAsync((void**)&out.edge_faces, sizeof(int64_t) * 2 * (size_t)(NO > 0 ? NO : 1), s)) !=
        cudaSuccess)
        return e;
    if (NO > 0) {
        k_edge_emit<<<nblk(NO), kBs, 0, s>>>(NO, a.face_offsets, a.face_verts, occ_face, own, eid, cnt, out.face_edges,
                                             out.edges, edge_cnt);
        note_launch();
    }
    if ((e = exscan_u32(edge_cnt, eoff, NE, s)) != cudaSuccess) return e;
    cudaMemsetAsync(fill, 0, sizeof(uint32_t) * (size_t)(NE > 0 ? NE : 1), s);
    if (NO > 0) {
        k_edge_fill<<<nblk(NO), kBs, 0, s>>>(NO, out.face_edges, eoff, fill, occ);
        note_launch();
    }
    if (NE > 0) {
        k_edge_sort<<<nblk(NE), kBs, 0, s>>>(NE, eoff, edge_cnt, occ, occ_face, a.face_offsets, out.edge_faces,
                                             out.edge_face_offsets);
        note_launch();
    }
    k_set_total<<<1, 1, 0, s>>>(out.edge_face_offsets, NE, NO);
    note_launch();
    // patches: faces linked through manifold edges
    int32_t* padj = pool.get<int32_t>(NO);
    if (pool.err) return pool.err;
    if (NO > 0) {
        k_patch_adj<<<nblk(NO), kBs, 0, s>>>(NO, out.face_edges, occ_face, eoff, edge_cnt, occ, padj);
        note_launch();
    }
    if ((e = ordered_bfs<int64_t>(NF, a.face_offsets, padj, nullptr, &out.patch_offsets, &out.n_patches,
                                  &out.patch_faces, status, pool, s)) != cudaSuccess)
        return e;
    if ((e = cudaMallocAsync((void**)&out.patch_labels, sizeof(int64_t) * 2 * (size_t)(out.n_patches > 0 ? out.n_patches : 1),
                             s)) != cudaSuccess)
        return e;
    if (out.n_patches > 0) {
        k_patch_labels<<<nblk(out.n_patches), kBs, 0, s>>>(out.n_patches, out.patch_offsets, out.patch_faces, a.face_func,
                                                           out.patch_labels);
        note_launch();
    }
    // chains: non-manifold edges linked through vertices with exactly two of them
    uint32_t* nm_flag = pool.get<uint32_t>(NE);
    uint32_t* nm_id = pool.get<uint32_t>(NE);
    uint32_t* vcnt = pool.get<uint32_t>(a.n_verts);
    int32_t* vedge = pool.get<int32_t>(2 * a.n_verts);
    if (pool.err) return pool.err;
    if (NE > 0) {
        k_nm_mark<<<nblk(NE), kBs, 0, s>>>(NE, edge_cnt, nm_flag);
        note_launch();
    }
    if ((e = exscan_u32(nm_flag, nm_id, NE, s)) != cudaSuccess) return e;
    int64_t NM = 0;
    if ((e = scan_total(nm_flag, nm_id, NE, &NM, s)) != cudaSuccess) return e;
    out.n_nm_edges = NM;
    int32_t* cadj = pool.get<int32_t>(2 * NM);
    int64_t* cadj_off = pool.get<int64_t>(NM + 1);
    int64_t* nm_edge = pool.get<int64_t>(NM);
    if (pool.err) return pool.err;
    cudaMemsetAsync(vcnt, 0, sizeof(uint32_t) * (size_t)(a.n_verts > 0 ? a.n_verts : 1), s);
    if (NE > 0) {
        k_nm_vert<<<nblk(NE), kBs, 0, s>>>(NE, nm_flag, nm_id, out.edges, vcnt, vedge);
        note_launch();
        k_chain_adj<<<nblk(NE), kBs, 0, s>>>(NE, nm_flag, nm_id, out.edges, vcnt, vedge, cadj, nm_edge);
        note_launch();
    }
    if (NM > 0) {
        k_iota2_i64<<<nblk(NM + 1), kBs, 0, s>>>(NM + 1, cadj_off);
        note_launch();
    }
    if ((e = ordered_bfs<int64_t>(NM, cadj_off, cadj, nm_edge, &out.chain_offsets, &out.n_chains, &out.chain_edges,
                                  status, pool, s)) != cudaSuccess)
        return e;
    uint32_t hs = 0;
    cudaMemcpyAsync(&hs, status, 4, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    if (hs) return cudaErrorUnknown;
    return cudaGetLastError();
}

}  // namespace ria
