// Host-side launchers of the device kernels (one declaration per kernel family).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/ria.h"

namespace ria {

// counts every kernel of this library as it is launched (ria_kernel_launches)
void note_launch();

struct IASum4 {  // IASummary / MISummary packed as 4 x u16 (MI: n_mi_v, n_mi_f, n_mi_loop, n_bnd_f)
    uint16_t a, b, c, d;
};

struct GridDesc {
    int64_t res;  // 0: explicit pts / tets
    double bmin[3], bmax[3];
};

// ---- stage a / b (k_ab.cu)
// grid coordinates per axis: coords[a * (res+1) + n]
void launch_grid_coords(const GridDesc& g, double* coords, cudaStream_t s);
// grid sampling fused with the per-vertex masks: IA -> (pos, neg) masks; MI -> (argmax mask, 0).
// tab: scratch of 6 * F * (res+1) doubles for the per-axis terms.
// tab: 6 N F per-axis terms; xy: N N F first sums per (x, y) column (scratch)
void launch_sample_grid(bool mi, const ria_function* d_funcs, int F, const GridDesc& g, const double* coords,
                        double* tab, double* xy, double* fv, ulonglong2* vmask, unsigned long long* n_zero,
                        cudaStream_t s);
// sampling at explicit points (vmask / n_zero may be null)
void launch_sample_points(const ria_function* d_funcs, int F, const double* pts, int64_t V, double* fv,
                          ulonglong2* vmask, unsigned long long* n_zero, cudaStream_t s);
void launch_vertex_masks(bool mi, const double* fv, int64_t V, int F, ulonglong2* vmask, unsigned long long* n_zero,
                         cudaStream_t s);

// ---- CSG pruning (k_extract.cu): per face of an implicit-arrangement mesh in [f0, f1): 0 not on the
// boundary of the shape, 1 inside on the positive side of the face's function, 2 on its negative
// side.  prog: postfix tokens (>= 0 function, -1 intersection, -2 union, -3 negation); nprog = 0: the
// union of all functions.  Function j is inside where its sign is positive (pos_inside) or negative.
struct CsgArgs {
    int64_t f0, f1;
    const int64_t* face_tet_offsets;
    const int64_t* face_tets;
    const int64_t* face_func;
    const uint32_t* act_tet;
    int64_t A;
    const uint64_t* act_desc;
    const uint64_t* act_mask;
    const uint8_t* heap;
    const uint8_t* heap_big;
    const uint8_t* table;
    const uint32_t* table_off;
    const double* fv;
    int F;                  // row stride of fv
    int nfunc;              // functions of the problem (F, or fewer in a batch)
    const int64_t* d_tets;  // explicit tets, or the grid of `res` cubes with ids offset by tbase / vbase
    int64_t res, tbase, vbase;
    const int32_t* prog;
    int nprog;
    int pos_inside;
    uint8_t* out;
    uint64_t* sides = nullptr;  // instead of labels: per face the sign vectors (bit j: function j > 0)
                                // on the positive and on the negative side of the face's function
};
void launch_csg(const CsgArgs& a, cudaStream_t s);

// ---- batched grids (k_ab.cu): many independent tet5 grids concatenated problem-major
struct BatchProblem {
    int64_t vbase, tbase;  // first vertex / tet of the problem in the batch numbering
    int32_t res, F;        // cubes per axis, functions
    int32_t foff, pad;     // first function in the concatenated function array
    double bmin[3], bmax[3];
};
// Grid points, values (stride Fmax; columns F..Fmax-1 hold a constant that is never active: +1 for
// the implicit arrangement, -inf for the material interface) and vertex masks of every problem.
// blk_off[p] is the first sampling block of problem p (n + 1 entries, blocks of kBatchSampleBlock
// vertices); n_zero_p receives each problem's degenerate-vertex count.
constexpr int kBatchSampleBlock = 128;
void launch_batch_sample(bool mi, const BatchProblem* probs, int n, const uint32_t* blk_off, uint32_t n_blocks,
                         const ria_function* funcs, int Fmax, double* pts, double* fv, ulonglong2* vmask,
                         unsigned long long* n_zero, unsigned long long* n_zero_p, cudaStream_t s);
// explicit tets of every problem (global vertex ids); tet_base[p] = probs[p].tbase, n + 1 entries
void launch_batch_tets(const BatchProblem* probs, const int64_t* tet_base, int n, int64_t T, int64_t* tets,
                       cudaStream_t s);
// per problem: first mesh vertex and first face (n + 1 entries each) and the active-tet statistics
// (active count, k histogram) from the active lists
void launch_batch_ranges(const int64_t* tet_base, int n, const int64_t* verts, int64_t n_verts,
                         const int64_t* face_tet_offsets, const int64_t* face_tets, int64_t n_faces,
                         int64_t* vert_first, int64_t* face_first, cudaStream_t s);
void launch_batch_active_stats(bool mi, const int64_t* tet_base, int n, const uint32_t* act_tet,
                               const uint64_t* act_mask, int64_t A, unsigned long long* stats4, cudaStream_t s);

// Ordered compaction of the active tets.  Pass 1 counts per block (active, generic) and the k
// histogram; pass 2 writes, in tet order, the active tets and the tets that need the generic cut.
// general-case tets are listed in bins of equal active-function count, the heaviest first: bin 0
// holds k >= kGenBins (+1 for MI), bin kGenBins-1 the lightest; the count kernel writes, per block,
// the active count and then one count per bin ([1 + kGenBins][blocks], scanned as one array)
constexpr int kGenBins = 8;
struct FilterOut {
    uint32_t* act_tet;    // [A]
    uint64_t* act_mask;   // [A] active functions (bit j = function j)
    uint64_t* act_desc;   // [A] record descriptor (lookup entries are filled here)
    IASum4* act_sum;      // [A]
    uint32_t* gen;        // [G] indices into the active arrays
};
// raises ST_BADINPUT if an explicit tet refers to a vertex outside 0..V-1
void launch_check_tets(const int64_t* d_tets, int64_t T, int64_t V, uint32_t* status, cudaStream_t s);
int64_t filter_num_blocks(int64_t T);
void launch_filter_count(bool mi, const ulonglong2* vmask, const double* fv, int F, const int64_t* d_tets,
                         const GridDesc& g, int64_t T, bool use_table, uint32_t* blk_counts /* [2][nblk] */,
                         unsigned long long* khist /* [3] */, cudaStream_t s);
void launch_filter_scatter(bool mi, const ulonglong2* vmask, const double* fv, int F, const int64_t* d_tets,
                           const GridDesc& g, int64_t T, bool use_table, const uint32_t* blk_offsets /* [2][nblk] */,
                           const IASum4* table_sum, FilterOut out, cudaStream_t s);

// ---- stage c (k_cut.cu)
struct WaitRec;
struct CutArgs {
    bool mi;
    const uint32_t* list;  // indices into the active arrays
    int64_t n;
    const uint32_t* act_tet;
    const uint64_t* act_mask;
    uint64_t* act_desc;
    IASum4* act_sum;
    const double* fv;
    int F;
    const int64_t* d_tets;
    GridDesc g;
    uint8_t* heap;
    unsigned long long* heap_used;
    uint64_t heap_cap;
    uint64_t desc_bit;           // or-ed into the descriptors written (0 or kBigHeapBit)
    uint32_t* deferred;          // fast variant: tets handed to the exact variant
    unsigned int* n_deferred;
    const unsigned int* n_dev = nullptr;  // when set, the list holds min(n, *n_dev) tets (a count on the device)
    // when set, a list of at most route_at tets goes to the warp kernel and a longer one to the
    // thread kernel (both are launched; the other returns at once)
    int64_t route_at = 0;
    unsigned int* next = nullptr;         // warp kernel: zeroed counter from which warps take tets in list order
    // launch shapes chosen by the tuning record (ria_tuning): resident blocks of the warp kernel per
    // SM (0: the occupancy limit) and threads per block of the thread kernel (0: from the tet count)
    int warp_blocks_per_sm = 0;
    int fast_block = 0;
    uint32_t* owners = nullptr;           // the lookup pass: tets that claimed their key (else in deferred)
    unsigned int* n_owners = nullptr;
    uint32_t* status;
    // explicit per-tet rows (the per-tet batch API): rows of tet i are value_off[i]..value_off[i+1]-1
    const double* values = nullptr;
    const uint32_t* value_off = nullptr;
    // one-plane lookup table (implicit arrangement), used for tets with one effective plane
    const uint8_t* table = nullptr;
    const uint32_t* table_off = nullptr;
    // secondary lookup (two planes / three materials): disabled when slots is null
    struct Cache {
        unsigned long long* slots = nullptr;  // (key + 1) << 32 | entry; 0 = empty
        uint32_t slot_mask = 0;
        uint32_t cap = 0;                     // entries
        unsigned long long* next = nullptr;   // entries taken (64-bit: never wraps)
        unsigned long long* heap_used = nullptr;
        uint64_t heap_base = 0, heap_cap = 0; // template bytes in the table region
        uint8_t* table = nullptr;             // the mode's table region (entries follow the 81 patterns)
        uint32_t* table_off = nullptr;
        IASum4* table_sum = nullptr;
        uint32_t gen = 0;                     // call number: claims of other calls can be taken over
    } cache;
    // the lookup pass: tets whose key another tet of this call claimed (resolved after the cuts)
    WaitRec* wait = nullptr;
    unsigned int* n_wait = nullptr;
};
// a tet waiting for the record of its key (secondary lookup), with what its own record needs
struct WaitRec {
    uint32_t ai;
    uint32_t key;
    uint8_t k, r0, r1, pad;
    uint8_t rep[8];
};
// tets the lookup tables finish without a cut (IA: one or two effective planes found in the table
// or the secondary cache; MI: three materials found in the cache); the others are appended, in list
// order per warp, to `deferred` for the cut kernels
void launch_cut_prep(const CutArgs& a, cudaStream_t s);
// fill the secondary lookup (a.cache) from synthetic configurations, once per process and mode
void launch_seed_cache(const CutArgs& a, cudaStream_t s);
// the waiting tets of the lookup pass, after the cuts have published their keys' records (a key
// still unpublished sends its tets to the deferred list)
void launch_cut_wait(const CutArgs& a, cudaStream_t s);
// implicit arrangement, one warp per tet with its state in shared memory (exact predicates); a tet
// beyond its capacity goes to the deferred list
// light: the smaller state (IAWarpCutLight: more resident warps per SM), for the light bins' leftovers
void launch_cut_warp(const CutArgs& a, cudaStream_t s, bool light = false);
// filtered variants, one thread per tet: `mid` for the heavy bins (four or more active functions,
// up to 16), the small one otherwise; a tet that outgrows them, or whose record does not fit the
// heap, goes to the deferred list
void launch_cut_fast(const CutArgs& a, cudaStream_t s, bool mid = false);
// material interface, tets with many materials: one thread per material's cell (filtered), merged per
// tet; tets it cannot finish go to the deferred list
void launch_cut_mi_split(const CutArgs& a, cudaStream_t s);
// first bin of tets for the small filtered variant (three or fewer active functions)
constexpr int kFirstSmallBin(bool mi) { return mi ? 6 : 5; }
// exact variant: one tet per block, state in shared memory
void launch_cut_big(const CutArgs& a, cudaStream_t s);
size_t cut_big_slot_bytes(bool mi);
// per-device lookup tables: IA one active plane, MI two active materials; 81 sign patterns each
constexpr int kTablePatterns = 81;
constexpr int kTableStride = 256;
// secondary lookup entries per mode and their template bytes (after the 81 patterns)
constexpr uint32_t kCacheEntries = 1u << 18;
constexpr uint32_t kCacheSlots = 1u << 20;
constexpr uint64_t kCacheHeapBytes = 64ull << 20;
void launch_build_table(bool mi, uint8_t* table, uint32_t* table_off, IASum4* table_sum, void* scratch,
                        uint32_t* status, cudaStream_t s);
// robust test: cut every listed tet with its rows in the given and in the reversed order with the
// exact variant; counts the tets whose vertex/face/cell counts differ
void launch_robust(const CutArgs& a, void* scratch, int64_t scratch_slots, unsigned long long* n_fail,
                   cudaStream_t s);

// A second stream of the current device for the calling thread, with events to fork work onto it
// and join it back (capi.cu); each thread runs one call at a time, so a call may use it freely.
struct AuxStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
cudaError_t aux_stream(AuxStream** out);
// 64 words of pinned host memory for the calling thread: counters copied there arrive while the
// stream keeps working (the copy into pageable memory would wait for the whole stream).
cudaError_t pinned_words(uint64_t** out);

// ---- stage d (k_extract.cu)
struct ExtractArgs {
    bool mi;
    int64_t A;
    const uint32_t* act_tet;
    const uint64_t* act_mask;
    const uint64_t* act_desc;
    const uint8_t* heap;
    const uint8_t* table;
    const uint32_t* table_off;
    const uint8_t* heap_big;
    const double* fv;
    int F;
    const int64_t* d_tets;
    const double* d_pts;
    const double* coords;  // grid coordinates per axis (grid inputs)
    GridDesc g;
    int64_t V;
    uint32_t* status;
    // implicit arrangement: dedup tables sized for the usual load, with bounded probing; an insert
    // that runs out raises ST_HASH_FULL and the caller runs the extraction again with tables sized
    // for the worst case (tight_tables = false)
    bool tight_tables = true;
};
struct ExtractOut {
    int64_t n_verts = 0, n_faces = 0, n_face_verts = 0, n_face_tets = 0;
    double* xyz = nullptr;
    int64_t* verts = nullptr;
    int64_t* face_offsets = nullptr;
    int64_t* face_verts = nullptr;
    int64_t* face_tet_offsets = nullptr;
    int64_t* face_tets = nullptr;
    int64_t* face_func = nullptr;
};
// Occurrence bases of the extraction (the exclusive scan of the per-tet counts of the cut; material
// interface: of its phase-0 counts), prepared before run_extract so that their totals come back with
// the cut stage's synchronization.  launch_extract_bases enqueues the scan into `buf`
// (extract_bases_bytes(A) device bytes) and writes the four totals (the counts' four fields) to the
// device counters `totals`; the caller copies them into ExtractBases::total.
// launch_table_summaries (implicit arrangement) summarises the table records the tets use (see the
// extraction's vertex pass), so that this work too is enqueued before the extraction is issued.
struct ExtractBases {
    const void* base = nullptr;
    uint64_t total[4] = {0, 0, 0, 0};
    uint32_t* tsum_state = nullptr;  // the table-record summaries, when prepared
    uint64_t* tsum = nullptr;
};
size_t extract_bases_bytes(int64_t A, bool summaries);
void launch_extract_bases(int64_t A, const IASum4* act_sum, void* buf, unsigned long long* totals, ExtractBases* out,
                          cudaStream_t s);
// the summaries, into the same buffer (sized with summaries = true), after launch_extract_bases
void launch_table_summaries(int64_t A, const uint64_t* act_desc, const uint8_t* table, const uint32_t* table_off,
                            void* buf, ExtractBases* out, cudaStream_t s);
// Runs the whole extraction; allocates the outputs with cudaMallocAsync on `s`.  `pre` (may be null):
// bases prepared by launch_extract_bases on the same records.
cudaError_t run_extract(const ExtractArgs& a, const IASum4* act_sum, const ExtractBases* pre, ExtractOut& out,
                        cudaStream_t s);

// ria_compute_arrangement_batch_noalloc (k_noalloc.cu): returns a ria_status value and a static
// message on failure; allocates nothing
int run_batch_noalloc(const double* d_values, const uint32_t* d_value_offsets, uint64_t n_tets, uint8_t* d_records,
                      uint64_t capacity, uint64_t* d_record_offsets, cudaStream_t s, const char** msg);

// local-to-global maps of a finished mesh (k_tetmaps.cu, RIA_MESH_TET_*): per record vertex its mesh
// vertex or -v-1, per record face its mesh face or -1, each a CRS over the tets
struct TetMapArgs {
    bool mi;
    int64_t A, T;
    const uint32_t* act_tet;
    const uint64_t* act_desc;
    const uint64_t* act_mask;
    const uint8_t* heap;
    const uint8_t* heap_big;
    const uint8_t* table;
    const uint32_t* table_off;
    const int64_t* d_tets;  // explicit tets, or nullptr for the grid of `res` cubes
    int64_t res;
    const int64_t* verts;   // mesh vertex records [n_verts][11]
    int64_t n_verts;
    const int64_t* face_tet_offsets;
    const int64_t* face_tets;
    int64_t n_faces;
};
// d_vert_offsets / d_face_offsets: [T + 1]; the maps are allocated with cudaMallocAsync on `s`;
// cudaErrorUnknown when the records and the mesh disagree
cudaError_t gather_tet_maps(const TetMapArgs& m, int64_t* d_vert_offsets, int64_t* d_face_offsets,
                            int64_t** d_tet_verts, int64_t* n_tet_verts, int64_t** d_tet_faces, int64_t* n_tet_faces,
                            cudaStream_t s);

// mesh connectivity (k_connect.cu): the reference's compute_mesh_edges, compute_patches and
// compute_chains over a finished mesh (RIA_MESH_EDGE*, RIA_MESH_PATCH*, RIA_MESH_CHAIN*)
struct ConnArgs {
    int64_t n_faces, n_face_verts, n_verts;
    const int64_t* face_offsets;
    const int64_t* face_verts;
    const int64_t* face_func;  // [n_faces][2]
};
struct ConnOut {
    int64_t n_edges = 0, n_patches = 0, n_chains = 0, n_nm_edges = 0;
    int64_t* edges = nullptr;              // [n_edges][2]
    int64_t* edge_face_offsets = nullptr;  // [n_edges + 1]
    int64_t* edge_faces = nullptr;         // [n_face_verts][2]: (face, local edge)
    int64_t* face_edges = nullptr;         // [n_face_verts]: edges_of_face, by face_offsets
    int64_t* patch_offsets = nullptr;      // [n_patches + 1]
    int64_t* patch_faces = nullptr;        // [n_faces]
    int64_t* patch_labels = nullptr;       // [n_patches][2]: func_index of the patch's first face
    int64_t* chain_offsets = nullptr;      // [n_chains + 1]
    int64_t* chain_edges = nullptr;        // [n_nm_edges]
};
// allocates the outputs with cudaMallocAsync on `s`; cudaErrorUnknown on an internal inconsistency
cudaError_t build_connectivity(const ConnArgs& a, ConnOut& out, cudaStream_t s);

// records in tet order (for RIA_MESH_REC_*)
cudaError_t gather_records(bool mi, int64_t A, int64_t T, const uint32_t* act_tet, const uint64_t* act_desc,
                           const uint8_t* heap, const uint8_t* heap_big, const uint8_t* table, const uint32_t* table_off,
                           int64_t* d_rec_offsets /* [T+1] */, uint8_t** d_rec_bytes, int64_t* n_bytes,
                           cudaStream_t s);
// CRS of the active functions (RIA_MESH_FUNC_IN_TET / START_INDEX)
cudaError_t gather_func_in_tet(int64_t A, int64_t T, const uint32_t* act_tet, const uint64_t* act_mask,
                               int64_t* d_start /* [T+1] */, int64_t** d_func_in_tet, int64_t* n_vals,
                               cudaStream_t s);

}  // namespace ria
