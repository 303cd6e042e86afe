// One material's cell of the material interface, clipped by a warp (the same cell as MICut::clip and
// MICut::export_cell, which one thread runs).
//
// A cell is the tet clipped, in material order, by the half-spaces m >= j of the other materials.
// Run by one thread, every clip step is a chain of dependent shared-memory accesses over the cell's
// vertices and faces, and a four- or five-material tet takes hundreds of thousands of cycles with
// nothing to hide the latency.  Here each step runs across the lanes, one lane per vertex or face:
//   A  the vertices referenced by the faces (live) and their signs against material j
//   B  the crossing edges of the faces, into a shared hash; one new vertex per edge, numbered by
//      slot, its labels and predicate cache built on its own lane
//   C  every face rebuilt with its new vertices: dropped when it has no negative vertex, else cut
//      to its non-positive part; scans give the kept faces' ids and loop offsets in face order
//   D  the cap face chained from the faces' cap edges (a successor table), appended last
// Vertex ids differ from the serial clip's (they follow the hash slots); faces, their order, their
// loops' vertex keys and loop orders are the serial clip's, so the merged record is the same bytes.
//
// `LanesG` is the cooperating group (cut_ia_warp.cuh): a warp on the device, one lane on the host,
// where every lane loop is the serial loop (the host build checks the algorithm against the oracle).
#pragma once
#include "cut_ia_warp.cuh"
#include "cut_mi.cuh"

namespace ria {

// Per tet, shared by the warps that clip its cells: the groups of identical materials (rep) and the
// materials without a cell (no_cell) or without effect as clippers (no_clip), as MICut::prepare.
struct MIPrep {
    uint8_t rep[64];
    uint64_t no_cell, no_clip;
    RIA_HD bool has_cell(int m) const { return rep[m - 4] == m && !(no_cell & bit64(m - 4)); }
};

template <class LT>
RIA_HDI void mi_prepare_lanes(const LT& L, const double* mt, int k, MIPrep& P) {
    // rep[i]: the smallest material with the same four values (it is its own representative)
    for (int i = L.lane; i < k; i += L.W) {
        const double* a = mt + 4 * i;
        uint8_t r = (uint8_t)(4 + i);
        for (int j = 0; j < i; ++j) {
            const double* b = mt + 4 * j;
            if (a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) {
                r = (uint8_t)(4 + j);
                break;
            }
        }
        P.rep[i] = r;
    }
    L.sync();
    uint64_t nc = 0, ncl = 0;
    for (int a = L.lane; a < k; a += L.W) {
        if (P.rep[a] != 4 + a) continue;
        const double* x = mt + 4 * a;
        for (int b = 0; b < k; ++b) {
            if (b == a || P.rep[b] != 4 + b) continue;
            const double* y = mt + 4 * b;
            if (y[0] >= x[0] && y[1] >= x[1] && y[2] >= x[2] && y[3] >= x[3]) {
                nc |= bit64(a);
                if (y[0] > x[0] && y[1] > x[1] && y[2] > x[2] && y[3] > x[3]) ncl |= bit64(a);
            }
        }
    }
    const uint64_t nc_all = ((uint64_t)L.or_all((unsigned)(nc >> 32)) << 32) | L.or_all((unsigned)nc);
    const uint64_t ncl_all = ((uint64_t)L.or_all((unsigned)(ncl >> 32)) << 32) | L.or_all((unsigned)ncl);
    if (L.lane == 0) {
        P.no_cell = nc_all;
        P.no_clip = ncl_all;
    }
    L.sync();
}

template <int PV, int PF, int PL>
struct MIWarpClip {
    static_assert(PV <= 255 && PF <= 255 && PL <= 65535, "ids");
    static constexpr int kSlots = 64;  // crossing edges of one clip step (a power of two)
    const double* mt;
    int nv, nf, cur, fail;
    uint64_t mask[PV];
    uint8_t clab[PV][4];
    VCache vc[PV];
    int8_t sg[PV];
    uint8_t live[PV];
    uint8_t fother[2][PF];
    uint16_t foff[2][PF], flen[2][PF];
    uint8_t loops[2][PL];
    // one clip step
    uint32_t eslot[kSlots];  // crossing edge key + 1 (u | w << 8, u < w); 0 = empty
    uint8_t evert[kSlots];
    uint32_t succ[PV];  // cap chain: head of the cap edge leaving each vertex (~0u: none)
    uint8_t chas[PF], cwa[PF], cwb[PF];
    uint8_t vid[PV];  // export: cell vertex id of each live vertex

    RIA_HD const double* row_of(int l) const { return mt + 4 * (l - 4); }
    RIA_HD void set_fail(int code) { fail = code; }

    RIA_HD bool build_cache(int v) {
        bool bound[4] = {false, false, false, false};
        const double* rows[4];
        int m = 0;
        for (int t = 0; t < 4; ++t) {
            const int l = clab[v][t];
            if (l < 4)
                bound[l] = true;
            else
                rows[m++] = row_of(l);
        }
        uint8_t S[4];
        int s = 0;
        for (int c = 0; c < 4; ++c)
            if (!bound[c]) S[s++] = (uint8_t)c;
        return vcache_build(vc[v], true, s, S, m, rows, false);
    }

    RIA_HD int query(int v, const double* q) const {
        const double* rows[4];
        int m = 0;
        for (int t = 0; t < 4; ++t)
            if (clab[v][t] >= 4) rows[m++] = row_of(clab[v][t]);
        return vcache_query(vc[v], q, rows, false);
    }

    RIA_HD int edge_vertex(int u, int w) const {
        const uint32_t key = (uint32_t)(u < w ? (u | (w << 8)) : (w | (u << 8))) + 1u;
        const uint32_t h = (key * 2654435761u) >> 26;
        for (int p = 0; p < kSlots; ++p) {
            const uint32_t s = eslot[(h + p) & (kSlots - 1)];
            if (s == key) return evert[(h + p) & (kSlots - 1)];
            if (s == 0) return -1;
        }
        return -1;
    }

    template <class LT>
    RIA_HDI void mark_live(const LT& L) {
        for (int v = L.lane; v < nv; v += L.W) live[v] = 0;
        L.sync();
        for (int f = L.lane; f < nf; f += L.W)
            for (int t = 0; t < flen[cur][f]; ++t) live[loops[cur][foff[cur][f] + t]] = 1;
        L.sync();
    }

    // The cell of material m (MICut::clip).  Returns CUT_OK (`empty` when it has no interior),
    // CUT_DEFER (capacity or a predicate the filters cannot decide) or CUT_FAIL.
    template <class LT>
    RIA_HDI int clip(const LT& L, const double* mats, int k, const MIPrep& P, int m, bool& empty) {
        const int lane = L.lane;
        // the whole tet, labelled with material m
        for (int c = lane; c < 4; c += L.W) {
            int t = 0;
            for (int b = 0; b < 4; ++b)
                if (b != c) clab[c][t++] = (uint8_t)b;
            clab[c][3] = (uint8_t)m;
            mask[c] = (0xFull & ~bit64(c)) | bit64(m);
            fother[0][c] = (uint8_t)c;
            foff[0][c] = (uint16_t)(3 * c);
            flen[0][c] = 3;
            for (int j = 0; j < 3; ++j) loops[0][3 * c + j] = (uint8_t)tet_face_outward(c, j);
        }
        if (lane == 0) {
            mt = mats;
            nv = 4;
            nf = 4;
            cur = 0;
            fail = CUT_OK;
        }
        L.sync();
        for (int c = lane; c < 4; c += L.W)
            if (!build_cache(c)) set_fail(CUT_DEFER);
        L.sync();
        if (fail != CUT_OK) return fail;
        empty = false;
        for (int j = 4; j < 4 + k; ++j) {
            if (j == m || P.rep[j - 4] != j || (P.no_clip & bit64(j - 4))) continue;
            const double* qv = row_of(j);
            const int nv0 = nv, nf0 = nf, nb = cur ^ 1;
            // A: live vertices and their signs
            mark_live(L);
            bool hp = false, hn = false;
            for (int v = lane; v < nv0; v += L.W) {
                sg[v] = 0;
                if (!live[v]) continue;
                const int s = query(v, qv);
                if (s == 2) {
                    set_fail(CUT_DEFER);
                    continue;
                }
                sg[v] = (int8_t)s;
                if (s == 0) mask[v] |= bit64(j);
                hp = hp || s > 0;
                hn = hn || s < 0;
            }
            for (int t = lane; t < kSlots; t += L.W) eslot[t] = 0;
            hp = L.or_all(hp ? 1u : 0u) != 0;
            hn = L.or_all(hn ? 1u : 0u) != 0;
            L.sync();
            if (fail != CUT_OK) return fail;
            if (!hn) {
                empty = true;
                break;
            }
            if (!hp) continue;
            // B: crossing edges into the hash, then one new vertex per edge, numbered by slot
            for (int f = lane; f < nf0; f += L.W) {
                const int Lf = flen[cur][f];
                for (int t = 0; t < Lf; ++t) {
                    const int u = loops[cur][foff[cur][f] + t];
                    const int w = loops[cur][foff[cur][f] + (t + 1 == Lf ? 0 : t + 1)];
                    if (sg[u] * sg[w] >= 0) continue;
                    const uint32_t key = (uint32_t)(u < w ? (u | (w << 8)) : (w | (u << 8))) + 1u;
                    const uint32_t h = (key * 2654435761u) >> 26;
                    bool placed = false;
                    for (int p = 0; p < kSlots && !placed; ++p) {
                        uint32_t* slot = &eslot[(h + p) & (kSlots - 1)];
#if defined(__CUDA_ARCH__)
                        const uint32_t old = atomicCAS(slot, 0u, key);
#else
                        const uint32_t old = *slot;
                        if (old == 0) *slot = key;
#endif
                        placed = old == 0 || old == key;
                    }
                    if (!placed) set_fail(CUT_DEFER);
                }
            }
            L.sync();
            if (fail != CUT_OK) return fail;
            int added = 0;
            for (int base = 0; base < kSlots; base += L.W) {
                const int t = base + lane;
                const uint32_t key = t < kSlots ? eslot[t] : 0u;
                const unsigned bm = L.ballot(key != 0);
                if (key) {
                    const int id = nv0 + added + L.below(bm);
                    if (id >= PV) {
                        set_fail(CUT_DEFER);
                    } else {
                        evert[t] = (uint8_t)id;
                        const int u = (int)((key - 1u) & 0xFF), w = (int)((key - 1u) >> 8);
                        const uint64_t em = mask[u] & mask[w];
                        const uint64_t nm = em | bit64(j);
                        mask[id] = nm;
                        sg[id] = 0;
                        if (popc64(em) != 3) {
                            set_fail(CUT_DEFER);  // more than four tight labels: an exact rank test
                        } else {
                            int c = 0;
                            for (int l = 0; l < 64 && c < 4; ++l)
                                if (nm & bit64(l)) clab[id][c++] = (uint8_t)l;
                            if (!build_cache(id)) set_fail(CUT_DEFER);
                        }
                    }
                }
                added += L.count(bm);
            }
            L.sync();
            if (fail != CUT_OK) return fail;
            // C: faces rebuilt in face order
            int kept_base = 0, used = 0;
            for (int base = 0; base < nf0; base += L.W) {
                const int f = base + lane;
                uint8_t full[PV + 8];
                int n = 0, cnt = 0;
                bool keep = false, fp = false;
                if (f < nf0) {
                    chas[f] = 0;
                    const int Lf = flen[cur][f];
                    bool fn = false;
                    for (int t = 0; t < Lf; ++t) {
                        const int u = loops[cur][foff[cur][f] + t];
                        const int w = loops[cur][foff[cur][f] + (t + 1 == Lf ? 0 : t + 1)];
                        if (n >= PV + 8) {
                            set_fail(CUT_DEFER);
                            break;
                        }
                        full[n++] = (uint8_t)u;
                        fp = fp || sg[u] > 0;
                        fn = fn || sg[u] < 0;
                        if (sg[u] * sg[w] < 0) {
                            const int e = edge_vertex(u, w);
                            if (e < 0 || n >= PV + 8) {
                                set_fail(CUT_DEFER);
                                break;
                            }
                            full[n++] = (uint8_t)e;
                        }
                    }
                    keep = fn && fail == CUT_OK;
                    if (keep) {
                        int j0 = -1;
                        for (int t = 0; t < n; ++t) {
                            const int prev = full[t == 0 ? n - 1 : t - 1];
                            if (sg[full[t]] < 0 && sg[prev] >= 0) {
                                j0 = t;
                                break;
                            }
                        }
                        if (j0 >= 0) {
                            int j1 = j0;
                            while (sg[full[(j1 + 1) % n]] < 0) j1 = (j1 + 1) % n;
                            const int wa = full[(j0 - 1 + n) % n], wb = full[(j1 + 1) % n];
                            if (wa != wb) {
                                chas[f] = 1;
                                cwa[f] = (uint8_t)wa;
                                cwb[f] = (uint8_t)wb;
                            }
                        }
                        for (int t = 0; t < n; ++t) cnt += !(fp && sg[full[t]] > 0);
                    }
                }
                int tot = 0;
                const int off = L.scan(keep ? cnt : 0, tot);
                const unsigned km = L.ballot(keep);
                const int g = kept_base + L.below(km);
                if (used + tot > PL || kept_base + L.count(km) >= PF) set_fail(CUT_DEFER);
                if (keep && used + tot <= PL && g < PF) {
                    int w = used + off;
                    fother[nb][g] = fother[cur][f];
                    foff[nb][g] = (uint16_t)w;
                    flen[nb][g] = (uint16_t)cnt;
                    for (int t = 0; t < n; ++t)
                        if (!(fp && sg[full[t]] > 0)) loops[nb][w++] = full[t];
                }
                kept_base += L.count(km);
                used += tot;
            }
            for (int v = lane; v < PV; v += L.W) succ[v] = ~0u;
            L.sync();
            if (fail != CUT_OK) return fail;
            // D: the cap face, chained from the cap edges of the kept faces (which are the faces with
            // a negative vertex, the only ones with a cap edge)
            int nedge = 0, first = -1;
            for (int base = 0; base < nf0; base += L.W) {
                const int f = base + lane;
                const bool has = f < nf0 && chas[f];
                if (has) {
#if defined(__CUDA_ARCH__)
                    const uint32_t old = atomicCAS(&succ[cwa[f]], ~0u, (uint32_t)cwb[f]);
#else
                    const uint32_t old = succ[cwa[f]];
                    if (old == ~0u) succ[cwa[f]] = cwb[f];
#endif
                    if (old != ~0u) set_fail(CUT_DEFER);  // two cap edges leave one vertex
                }
                const unsigned hm = L.ballot(has);
#if defined(__CUDA_ARCH__)
                if (first < 0 && hm) first = cwa[base + __ffs(hm) - 1];
#else
                if (first < 0 && hm) first = cwa[f];
#endif
                nedge += L.count(hm);
            }
            L.sync();
            if (fail != CUT_OK) return fail;
            if (nedge < 3) return CUT_FAIL;
            if (kept_base >= PF || used + nedge > PL) return CUT_DEFER;
            if (lane == 0) {
                int curv = first;
                for (int t = 0; t < nedge && fail == CUT_OK; ++t) {
                    loops[nb][used + t] = (uint8_t)curv;
                    const uint32_t nxt = succ[curv];
                    if (nxt == ~0u)
                        fail = CUT_FAIL;
                    else
                        curv = (int)nxt;
                }
                if (fail == CUT_OK && curv != first) fail = CUT_FAIL;
                fother[nb][kept_base] = (uint8_t)j;
                foff[nb][kept_base] = (uint16_t)used;
                flen[nb][kept_base] = (uint16_t)nedge;
                nf = kept_base + 1;
                nv = nv0 + added;
                cur = nb;
            }
            L.sync();
            if (fail != CUT_OK) return fail;
        }
        return CUT_OK;
    }

    // The clipped polytope as a cell (MICut::export_cell): live vertices in id order with their keys
    // (four sorted labels), faces in order with loops over the cell's vertex ids.
    template <class LT, class Cell>
    RIA_HDI int export_cell(const LT& L, Cell& out) {
        mark_live(L);
        int n = 0;
        for (int base = 0; base < nv; base += L.W) {
            const int v = base + L.lane;
            const bool lv = v < nv && live[v];
            const unsigned bm = L.ballot(lv);
            if (lv) {
                const int id = n + L.below(bm);
                const uint64_t mk = mask[v];
                if (popc64(mk) != 4 || id >= Cell::kV) {
                    set_fail(CUT_DEFER);  // more than four tight labels: an exact rank test
                } else {
                    uint8_t lb[4];
                    int c = 0;
                    for (int l = 0; l < 64 && c < 4; ++l)
                        if (mk & bit64(l)) lb[c++] = (uint8_t)l;
                    out.vkey[id] = ((uint32_t)lb[0] << 24) | ((uint32_t)lb[1] << 16) | ((uint32_t)lb[2] << 8) | lb[3];
                    vid[v] = (uint8_t)id;
                }
            }
            n += L.count(bm);
        }
        L.sync();
        if (fail != CUT_OK) return fail;
        if (nf > Cell::kF) return CUT_DEFER;
        const int total = foff[cur][nf - 1] + flen[cur][nf - 1];
        if (total > Cell::kL) return CUT_DEFER;
        for (int f = L.lane; f < nf; f += L.W) {
            out.fother[f] = fother[cur][f];
            out.flen[f] = (uint8_t)flen[cur][f];
        }
        for (int t = L.lane; t < total; t += L.W) out.loops[t] = vid[loops[cur][t]];
        if (L.lane == 0) {
            out.nv = (uint8_t)n;
            out.nf = (uint8_t)nf;
        }
        L.sync();
        return CUT_OK;
    }
};

}  // namespace ria
