// Per-tet implicit arrangement on fixed-capacity state (one thread per tet).
//
// Replaces simplicial_arrangement::compute_arrangement (third-party, absent), called by the
// reference at src/implicit_arrangement.cpp:279,283 for each tet with the corner values of its
// active functions (:266-274).  Plane ids: 0..3 are the tet faces (face b is opposite corner b),
// implicit plane i is 4+i (src/extract_mesh.cpp:103-105).
//
// Algorithm: planes that are exact multiples of an earlier plane (or of a tet face) are grouped
// and skipped; every other plane splits each cell it crosses.  Signs come from exact predicates
// (exact.cuh).  A vertex created on edge (u, v) by plane q is labelled by the two smallest planes
// through both u and v plus q, which is the lexicographically smallest independent set of the
// planes through it.  The output is the canonical record documented in include/ria.h.
#pragma once
#include "exact.cuh"

namespace ria {

enum : int { CUT_OK = 0, CUT_DEFER = 1, CUT_FAIL = 2 };
constexpr uint8_t kNoCell = 0xFF;

RIA_HD uint64_t bit64(int l) { return uint64_t(1) << l; }
RIA_HD int popc64u(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
RIA_HD int ctz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

// A set of cells (ids below N), one 64-bit word per 64 cells.
template <int N>
struct CellSet {
    uint64_t w[(N + 63) / 64];
    RIA_HD void clear() {
        for (int i = 0; i < (N + 63) / 64; ++i) w[i] = 0;
    }
    RIA_HD void set(int c) { w[c >> 6] |= uint64_t(1) << (c & 63); }
    RIA_HD bool test(int c) const { return (w[c >> 6] >> (c & 63)) & 1; }
    RIA_HD void meet(const CellSet& a, const CellSet& b) {
        for (int i = 0; i < (N + 63) / 64; ++i) w[i] = a.w[i] & b.w[i];
    }
    RIA_HD bool any() const {
        uint64_t o = 0;
        for (int i = 0; i < (N + 63) / 64; ++i) o |= w[i];
        return o != 0;
    }
};

// Tet face b is opposite corner b; loops run counter-clockwise seen from inside the tet in the
// reference frame x = (P1, P2, P3).
RIA_HD int tet_face_inward(int b, int j) {
    const uint8_t t[4][3] = {{1, 3, 2}, {0, 2, 3}, {0, 3, 1}, {0, 1, 2}};
    return t[b][j];
}
RIA_HD int tet_face_outward(int b, int j) {
    const uint8_t t[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
    return t[b][j];
}

// Counts that the mesh extraction needs for one record.
struct IASummary {
    uint16_t n_iso_v;     // vertices on an iso face
    uint16_t n_iso_f;     // iso faces
    uint16_t n_iso_loop;  // total loop length of the iso faces
    uint16_t n_bnd_f;     // iso faces on the tet boundary
};

// Group coincident planes: rep[i] is 0xFF for the zero plane, the tet face b for a plane with a
// single nonzero corner value (a multiple of face b), the first earlier plane it is an exact multiple
// of, or 4+i.  Returns the number of planes that remain (rep[i] == 4+i); `first` is the first one.
RIA_HD int ia_group_planes(const double* pl, int k, uint8_t* rep, int& first) {
    int eff = 0;
    first = -1;
    for (int i = 0; i < k; ++i) {
        const double* a = pl + 4 * i;
        int nz = 0, last = -1;
        for (int c = 0; c < 4; ++c)
            if (a[c] != 0.0) {
                ++nz;
                last = c;
            }
        if (nz == 0) {
            rep[i] = 0xFF;
            continue;
        }
        if (nz == 1) {
            rep[i] = (uint8_t)last;
            continue;
        }
        rep[i] = (uint8_t)(4 + i);
        for (int j = 0; j < i; ++j) {
            if (rep[j] != 4 + j) continue;
            const double* b = pl + 4 * j;
            bool prop = true;
            for (int x = 0; x < 4 && prop; ++x)
                for (int y = x + 1; y < 4 && prop; ++y)
                    if (!prod_eq(a[x], b[y], a[y], b[x])) prop = false;
            if (prop) {
                rep[i] = (uint8_t)(4 + j);
                break;
            }
        }
        if (rep[i] == 4 + i) {
            if (first < 0) first = i;
            ++eff;
        }
    }
    return eff;
}

// Sign pattern of one plane: sum over corners of (s_c + 1) 3^c.
RIA_HD int ia_sign_pattern(const double* p) {
    int q = 0, w = 1;
    for (int c = 0; c < 4; ++c) {
        q += ((p[c] > 0.0) ? 2 : (p[c] < 0.0 ? 0 : 1)) * w;
        w *= 3;
    }
    return q;
}

RIA_HD int rd16h(const uint8_t* p) { return p[0] | (p[1] << 8); }

// Size of the record built by ia_record_from_template for a tet with k planes.
RIA_HD int ia_template_record_size(const uint8_t* tmpl, int k) {
    int nv = rd16h(tmpl + 2), nf = rd16h(tmpl + 4), nc = rd16h(tmpl + 6), nl = rd16h(tmpl + 8);
    return 10 + k + 3 * nv + 8 * nf + 2 * nl + 8 * nc;
}

// Extraction counts of an implicit-arrangement record (vertex ids below 256).  With `rep_of` set,
// the iso faces are those of a tet with groups rep_of[0 .. k_of) (a relabelled template: its own
// plane labels above 3 stay above 3, and only the tet faces' iso status follows the tet's groups).
RIA_HD void ia_record_summary(const uint8_t* b, IASummary& sum, const uint8_t* rep_of = nullptr, int k_of = 0) {
    const int kb = b[1], nv = rd16h(b + 2), nf = rd16h(b + 4);
    const uint8_t* rep = rep_of ? rep_of : b + 10;
    const int k = rep_of ? k_of : kb;
    const uint8_t* faces = b + 10 + kb + 3 * nv;
    const uint8_t* loops = faces + 8 * nf;
    uint64_t iso[4] = {0, 0, 0, 0};
    int nisof = 0, nloop = 0, nbnd = 0, off = 0;
    for (int f = 0; f < nf; ++f) {
        const int p = faces[8 * f];
        const int L = rd16h(faces + 8 * f + 6);
        bool is = p > 3;
        for (int j = 0; j < k && !is; ++j) is = rep[j] == p;
        if (is) {
            ++nisof;
            nloop += L;
            if (faces[8 * f + 1] & 1) ++nbnd;
            for (int t = 0; t < L; ++t) {
                int v = rd16h(loops + 2 * (off + t));
                iso[v >> 6] |= 1ull << (v & 63);
            }
        }
        off += L;
    }
    int niso = 0;
    for (int w = 0; w < 4; ++w) niso += popc64u(iso[w]);
    sum.n_iso_v = (uint16_t)niso;
    sum.n_iso_f = (uint16_t)nisof;
    sum.n_iso_loop = (uint16_t)nloop;
    sum.n_bnd_f = (uint16_t)nbnd;
}

// Destinations of the template relabels, written front to back: bytes, or (device, 8-byte aligned
// destination) 8-byte words assembled in a register.
struct ByteSink {
    uint8_t* d;
    RIA_HD void put(uint8_t b) { *d++ = b; }
    RIA_HD void flush() {}
};
struct WordSink {
    uint64_t* d;
    uint64_t acc = 0;
    int n = 0;
    RIA_HD void put(uint8_t b) {
        acc |= (uint64_t)b << (8 * n);
        if (++n == 8) {
            *d++ = acc;
            acc = 0;
            n = 0;
        }
    }
    RIA_HD void flush() {
        if (n) *d = acc;  // the rest of the last word is padding of the 8-byte allocation
    }
};

// The record of a tet whose planes all coincide with one plane i (or with tet faces / zero when
// eff == 0): the one-plane table entry `tmpl` of plane i's sign pattern with plane label 4 renamed
// 4+i, the cell sign bit moved accordingly, and the tet's own groups.  Equal to what the generic cut
// produces, since that cut skips every plane grouped with an earlier one.
template <class Sink>
RIA_HD void ia_template_relabel1(const uint8_t* tmpl, int k, const uint8_t* rep, int eff, int i, Sink& out) {
    const int nv = rd16h(tmpl + 2), nf = rd16h(tmpl + 4), nc = rd16h(tmpl + 6), nl = rd16h(tmpl + 8);
    const uint8_t lab = (uint8_t)(4 + (eff ? i : 0));
    out.put(tmpl[0]);
    out.put((uint8_t)k);
    for (int t = 2; t < 10; ++t) out.put(tmpl[t]);
    for (int j = 0; j < k; ++j) out.put(rep[j]);
    const uint8_t* s = tmpl + 11;
    for (int t = 0; t < 3 * nv; ++t) out.put(s[t] == 4 ? lab : s[t]);
    s += 3 * nv;
    for (int f = 0; f < nf; ++f)
        for (int t = 0; t < 8; ++t) out.put((t == 0 && s[8 * f] == 4) ? lab : s[8 * f + t]);
    s += 8 * nf;
    for (int t = 0; t < 2 * nl; ++t) out.put(s[t]);
    s += 2 * nl;
    for (int c = 0; c < nc; ++c) {
        uint64_t sig = 0;
        for (int t = 0; t < 8; ++t) sig |= (uint64_t)s[8 * c + t] << (8 * t);
        sig = eff ? ((sig & 16ull) ? (1ull << lab) : 0ull) : 0ull;
        for (int t = 0; t < 8; ++t) out.put((uint8_t)((sig >> (8 * t)) & 0xFF));
    }
    out.flush();
}

RIA_HD void ia_record_from_template(const uint8_t* tmpl, int k, const uint8_t* rep, int eff, int i, uint8_t* dst) {
    ByteSink o{dst};
    ia_template_relabel1(tmpl, k, rep, eff, i, o);
}

// The record of a tet whose planes reduce to two groups with representatives r1 < r2 (local
// indices): the canonical record `tmpl` of the two representative planes alone (k = 2, labels 4 and
// 5) with 4 renamed 4+r1 and 5 renamed 4+r2, the cell sign bits moved accordingly, and the tet's own
// groups.  The renaming keeps every order the canonical form sorts by, and the generic cut inserts
// exactly the representatives, so the result equals the generic cut's record.
template <class Sink>
RIA_HD void ia_template_relabel2(const uint8_t* tmpl, int k, const uint8_t* rep, int r1, int r2, Sink& out) {
    const int nv = rd16h(tmpl + 2), nf = rd16h(tmpl + 4), nc = rd16h(tmpl + 6), nl = rd16h(tmpl + 8);
    const uint8_t l1 = (uint8_t)(4 + r1), l2 = (uint8_t)(4 + r2);
    auto ren = [&](uint8_t x) -> uint8_t { return x == 4 ? l1 : (x == 5 ? l2 : x); };
    out.put(tmpl[0]);
    out.put((uint8_t)k);
    for (int t = 2; t < 10; ++t) out.put(tmpl[t]);
    for (int j = 0; j < k; ++j) out.put(rep[j]);
    const uint8_t* s = tmpl + 12;
    for (int t = 0; t < 3 * nv; ++t) out.put(ren(s[t]));
    s += 3 * nv;
    for (int f = 0; f < nf; ++f)
        for (int t = 0; t < 8; ++t) out.put(t == 0 ? ren(s[8 * f]) : s[8 * f + t]);
    s += 8 * nf;
    for (int t = 0; t < 2 * nl; ++t) out.put(s[t]);
    s += 2 * nl;
    for (int c = 0; c < nc; ++c) {
        uint64_t sig = 0;
        for (int t = 0; t < 8; ++t) sig |= (uint64_t)s[8 * c + t] << (8 * t);
        const uint64_t o = ((sig >> 4) & 1 ? (1ull << l1) : 0ull) | ((sig >> 5) & 1 ? (1ull << l2) : 0ull);
        for (int t = 0; t < 8; ++t) out.put((uint8_t)((o >> (8 * t)) & 0xFF));
    }
    out.flush();
}

RIA_HD void ia_record_from_template2(const uint8_t* tmpl, int k, const uint8_t* rep, int r1, int r2, uint8_t* dst) {
    ByteSink o{dst};
    ia_template_relabel2(tmpl, k, rep, r1, r2, o);
}

template <int MV, int MF, int MC, int ML, bool EXACT>
struct IACut {
    const double* pl;  // k x 4 corner values
    int k;
    uint8_t rep[64];
    int nv;
    uint8_t lab[MV][3];
    uint64_t mask[MV];
    VCache vc[MV];
    int8_t sg[MV];
    int nf;
    uint8_t fsupp[MF], fpos[MF], fneg[MF];
    uint16_t foff[MF], flen[MF];
    uint8_t loops[2][ML];
    int cur, lused;
    int nc;
    uint64_t csign[MC];

    RIA_HD void rows_of(int v, const double** rows, int& m) const {
        m = 0;
        for (int t = 0; t < 3; ++t)
            if (lab[v][t] >= 4) rows[m++] = pl + 4 * (lab[v][t] - 4);
    }

    RIA_HD bool build_cache(int v) {
        bool bound[4] = {false, false, false, false};
        const double* rows[3];
        int m = 0;
        for (int t = 0; t < 3; ++t) {
            int l = lab[v][t];
            if (l < 4)
                bound[l] = true;
            else
                rows[m++] = pl + 4 * (l - 4);
        }
        uint8_t S[4];
        int s = 0;
        for (int c = 0; c < 4; ++c)
            if (!bound[c]) S[s++] = (uint8_t)c;
        return vcache_build(vc[v], false, s, S, m, rows, EXACT);
    }

    RIA_HD int query(int v, const double* q) const {
        const double* rows[3];
        int m;
        rows_of(v, rows, m);
        return vcache_query(vc[v], q, rows, EXACT);
    }

    RIA_HD void group_planes() {
        int first;
        ia_group_planes(pl, k, rep, first);
    }

    // Returns CUT_OK, CUT_DEFER (fast variant: filter undecided or out of capacity) or CUT_FAIL.
    RIA_HDI int run(const double* planes, int kk) {
        const int kBad = EXACT ? CUT_FAIL : CUT_DEFER;
        pl = planes;
        k = kk;
        if (k > 60) return CUT_FAIL;
        group_planes();
        nv = 4;
        for (int c = 0; c < 4; ++c) {
            int t = 0;
            for (int b = 0; b < 4; ++b)
                if (b != c) lab[c][t++] = (uint8_t)b;
            mask[c] = 0xFull & ~bit64(c);
            if (!build_cache(c)) return kBad;
        }
        nf = 4;
        cur = 0;
        lused = 12;
        for (int b = 0; b < 4; ++b) {
            fsupp[b] = (uint8_t)b;
            fpos[b] = 0;
            fneg[b] = kNoCell;
            foff[b] = (uint16_t)(3 * b);
            flen[b] = 3;
            for (int j = 0; j < 3; ++j) loops[0][3 * b + j] = (uint8_t)tet_face_inward(b, j);
        }
        nc = 1;
        csign[0] = 0;

        for (int i = 0; i < k; ++i) {
            if (rep[i] != 4 + i) continue;
            const int q = 4 + i;
            const double* qv = pl + 4 * i;
            for (int v = 0; v < nv; ++v) {
                int s = query(v, qv);
                if (s == 2) return kBad;
                sg[v] = (int8_t)s;
                if (s == 0) mask[v] |= bit64(q);
            }
            CellSet<MC> cpos, cneg, strad;
            cpos.clear();
            cneg.clear();
            for (int f = 0; f < nf; ++f) {
                bool hp = false, hn = false;
                for (int j = 0; j < flen[f]; ++j) {
                    int s = sg[loops[cur][foff[f] + j]];
                    hp = hp || s > 0;
                    hn = hn || s < 0;
                }
                if (hp) {
                    cpos.set(fpos[f]);
                    if (fneg[f] != kNoCell) cpos.set(fneg[f]);
                }
                if (hn) {
                    cneg.set(fpos[f]);
                    if (fneg[f] != kNoCell) cneg.set(fneg[f]);
                }
            }
            strad.meet(cpos, cneg);
            for (int c = 0; c < nc; ++c)
                if (!strad.test(c) && cpos.test(c)) csign[c] |= bit64(q);
            if (!strad.any()) continue;

            // new vertices on crossing edges
            int ne = 0;
            uint16_t ekey[MV];
            uint8_t eval[MV];
            for (int f = 0; f < nf; ++f) {
                const int L = flen[f];
                for (int j = 0; j < L; ++j) {
                    int u = loops[cur][foff[f] + j], w = loops[cur][foff[f] + (j + 1 == L ? 0 : j + 1)];
                    if (sg[u] * sg[w] >= 0) continue;
                    uint16_t key = (uint16_t)(u < w ? (u | (w << 8)) : (w | (u << 8)));
                    bool found = false;
                    for (int e = 0; e < ne; ++e)
                        if (ekey[e] == key) found = true;
                    if (found) continue;
                    if (nv >= MV || ne >= MV) return kBad;
                    uint64_t em = mask[u] & mask[w];
                    int p1 = ctz64(em);
                    int p2 = ctz64(em & ~bit64(p1));
                    lab[nv][0] = (uint8_t)p1;
                    lab[nv][1] = (uint8_t)p2;
                    lab[nv][2] = (uint8_t)q;
                    mask[nv] = em | bit64(q);
                    sg[nv] = 0;
                    if (!build_cache(nv)) return kBad;
                    ekey[ne] = key;
                    eval[ne] = (uint8_t)nv;
                    ++ne;
                    ++nv;
                }
            }
            auto edge_vertex = [&](int u, int w) -> int {
                uint16_t key = (uint16_t)(u < w ? (u | (w << 8)) : (w | (u << 8)));
                for (int e = 0; e < ne; ++e)
                    if (ekey[e] == key) return eval[e];
                return -1;
            };

            // rebuild loops; split straddling faces; record each face's cap edge
            const int nf0 = nf;
            int8_t fside[MF];
            uint8_t cwa[MF], cwb[MF];
            int8_t chas[MF];
            int nb = cur ^ 1;
            int used = 0;
            for (int f = 0; f < nf0; ++f) {
                const int L = flen[f];
                uint8_t full[MV + 8];
                int n = 0;
                bool hp = false, hn = false;
                for (int j = 0; j < L; ++j) {
                    int u = loops[cur][foff[f] + j], w = loops[cur][foff[f] + (j + 1 == L ? 0 : j + 1)];
                    if (n >= MV + 8) return kBad;
                    full[n++] = (uint8_t)u;
                    hp = hp || sg[u] > 0;
                    hn = hn || sg[u] < 0;
                    if (sg[u] * sg[w] < 0) {
                        if (n >= MV + 8) return kBad;
                        full[n++] = (uint8_t)edge_vertex(u, w);
                    }
                }
                // negative run and its bounding zero vertices
                chas[f] = 0;
                int j0 = -1;
                for (int j = 0; j < n; ++j) {
                    int prev = full[j == 0 ? n - 1 : j - 1];
                    if (sg[full[j]] < 0 && sg[prev] >= 0) {
                        j0 = j;
                        break;
                    }
                }
                int j1 = j0;
                if (j0 >= 0) {
                    while (sg[full[(j1 + 1) % n]] < 0) j1 = (j1 + 1) % n;
                    int wa = full[(j0 - 1 + n) % n], wb = full[(j1 + 1) % n];
                    if (wa != wb) {
                        chas[f] = 1;
                        cwa[f] = (uint8_t)wa;
                        cwb[f] = (uint8_t)wb;
                    }
                }
                if (hp && hn) {
                    fside[f] = 2;
                    if (nf >= MF) return kBad;
                    // positive part keeps id f, negative part becomes face nf
                    int lp = 0, ln = 0;
                    for (int j = 0; j < n; ++j) lp += sg[full[j]] >= 0;
                    for (int j = 0; j < n; ++j) ln += sg[full[j]] <= 0;
                    if (used + lp + ln > ML) return kBad;
                    foff[f] = (uint16_t)used;
                    flen[f] = (uint16_t)lp;
                    for (int j = 0; j < n; ++j)
                        if (sg[full[j]] >= 0) loops[nb][used++] = full[j];
                    int g = nf++;
                    fsupp[g] = fsupp[f];
                    fpos[g] = fpos[f];
                    fneg[g] = fneg[f];
                    foff[g] = (uint16_t)used;
                    flen[g] = (uint16_t)ln;
                    // start the negative part at wa
                    int jstart = (j0 - 1 + n) % n;
                    for (int t = 0; t < n; ++t) {
                        int v = full[(jstart + t) % n];
                        if (sg[v] <= 0) loops[nb][used++] = (uint8_t)v;
                    }
                } else {
                    fside[f] = hp ? 1 : -1;
                    if (used + n > ML) return kBad;
                    foff[f] = (uint16_t)used;
                    flen[f] = (uint16_t)n;
                    for (int j = 0; j < n; ++j) loops[nb][used++] = full[j];
                }
            }
            const int nf1 = nf;

            // split cells and build their cap faces
            uint8_t cneg_of[MC];
            const int nc0 = nc;
            for (int c = 0; c < nc0; ++c) {
                cneg_of[c] = kNoCell;
                if (!strad.test(c)) continue;
                if (nc >= MC) return kBad;
                cneg_of[c] = (uint8_t)nc;
                csign[nc] = csign[c];
                csign[c] |= bit64(q);
                ++nc;
            }
            for (int c = 0; c < nc0; ++c) {
                if (!strad.test(c)) continue;
                uint8_t et[MF], eh[MF];
                int nedge = 0;
                for (int f = 0; f < nf0; ++f) {
                    if (!chas[f]) continue;
                    if (fpos[f] != c && fneg[f] != c) continue;
                    if (nedge >= MF) return kBad;
                    if (fneg[f] == c) {  // loop is outward for c
                        et[nedge] = cwa[f];
                        eh[nedge] = cwb[f];
                    } else {
                        et[nedge] = cwb[f];
                        eh[nedge] = cwa[f];
                    }
                    ++nedge;
                }
                if (nedge < 3) return CUT_FAIL;  // an open cap cannot happen with exact signs
                if (nf >= MF || used + nedge > ML) return kBad;
                int g = nf++;
                fsupp[g] = (uint8_t)q;
                fpos[g] = (uint8_t)c;
                fneg[g] = cneg_of[c];
                foff[g] = (uint16_t)used;
                flen[g] = (uint16_t)nedge;
                int curv = et[0];
                for (int t = 0; t < nedge; ++t) {
                    loops[nb][used++] = (uint8_t)curv;
                    int nxt = -1;
                    for (int e = 0; e < nedge; ++e)
                        if (et[e] == curv) {
                            nxt = eh[e];
                            break;
                        }
                    if (nxt < 0) return CUT_FAIL;
                    curv = nxt;
                }
                if (curv != et[0]) return CUT_FAIL;
            }
            // cell references of faces on the negative side
            for (int f = 0; f < nf1; ++f) {
                if (f < nf0 && fside[f] != -1) continue;
                if (fpos[f] != kNoCell && cneg_of[fpos[f]] != kNoCell) fpos[f] = cneg_of[fpos[f]];
                if (fneg[f] != kNoCell && cneg_of[fneg[f]] != kNoCell) fneg[f] = cneg_of[fneg[f]];
            }
            cur = nb;
            lused = used;
        }
        return CUT_OK;
    }

    // ---- canonical form
    uint8_t vorder[MV], vnew[MV];
    uint8_t corder[MC], cnew[MC];
    uint16_t forder[MF];  // face ids exceed 8 bits in the exact variant
    int loop_total;

    RIA_HD uint32_t vkey(int v) const { return ((uint32_t)lab[v][0] << 16) | ((uint32_t)lab[v][1] << 8) | lab[v][2]; }

    // Sort key of a face: supporting plane, then its three smallest (renumbered) vertex ids.  Two
    // distinct faces on one plane share at most an edge, so the three smallest ids already order
    // them as the full sorted vertex lists would.
    RIA_HD uint32_t face_key(int f) const {
        uint32_t s0 = 0xFF, s1 = 0xFF, s2 = 0xFF;
        for (int j = 0; j < flen[f]; ++j) {
            uint32_t v = vnew[loops[cur][foff[f] + j]];
            if (v < s0) {
                s2 = s1;
                s1 = s0;
                s0 = v;
            } else if (v < s1) {
                s2 = s1;
                s1 = v;
            } else if (v < s2) {
                s2 = v;
            }
        }
        return ((uint32_t)fsupp[f] << 24) | (s0 << 16) | (s1 << 8) | s2;
    }

    RIA_HDI void canonicalize() {
        // live vertices (referenced by a face) sorted by label
        uint8_t live[MV];
        for (int v = 0; v < nv; ++v) live[v] = 0;
        for (int f = 0; f < nf; ++f)
            for (int j = 0; j < flen[f]; ++j) live[loops[cur][foff[f] + j]] = 1;
        int n = 0;
        for (int v = 0; v < nv; ++v)
            if (live[v]) vorder[n++] = (uint8_t)v;
        for (int x = 1; x < n; ++x)
            for (int y = x; y > 0 && vkey(vorder[y - 1]) > vkey(vorder[y]); --y) {
                uint8_t t = vorder[y];
                vorder[y] = vorder[y - 1];
                vorder[y - 1] = t;
            }
        for (int i = 0; i < n; ++i) vnew[vorder[i]] = (uint8_t)i;
        nv_live = n;
        for (int c = 0; c < nc; ++c) corder[c] = (uint8_t)c;
        for (int x = 1; x < nc; ++x)
            for (int y = x; y > 0 && csign[corder[y - 1]] > csign[corder[y]]; --y) {
                uint8_t t = corder[y];
                corder[y] = corder[y - 1];
                corder[y - 1] = t;
            }
        for (int i = 0; i < nc; ++i) cnew[corder[i]] = (uint8_t)i;
        uint32_t fkey[MF];
        for (int f = 0; f < nf; ++f) {
            forder[f] = (uint16_t)f;
            fkey[f] = face_key(f);
        }
        for (int x = 1; x < nf; ++x)
            for (int y = x; y > 0 && fkey[forder[y - 1]] > fkey[forder[y]]; --y) {
                uint16_t t = forder[y];
                forder[y] = forder[y - 1];
                forder[y - 1] = t;
            }
        loop_total = 0;
        for (int f = 0; f < nf; ++f) loop_total += flen[f];
    }
    int nv_live;

    RIA_HD int record_size() const { return 10 + k + 3 * nv_live + 8 * nf + 2 * loop_total + 8 * nc; }

    // supporting plane carries an implicit function (the plane itself, or a tet face made
    // coplanar by an implicit plane)
    RIA_HD bool plane_is_iso(int p) const {
        if (p > 3) return true;
        for (int j = 0; j < k; ++j)
            if (rep[j] == p) return true;
        return false;
    }

    // Write the canonical record to dst (record_size() bytes) and the extraction summary.
    RIA_HDI void emit(uint8_t* dst, IASummary& sum) const {
        int o = 0;
        auto w8 = [&](int v) { dst[o++] = (uint8_t)v; };
        auto w16 = [&](int v) {
            dst[o++] = (uint8_t)(v & 0xFF);
            dst[o++] = (uint8_t)((v >> 8) & 0xFF);
        };
        w8(1);
        w8(k);
        w16(nv_live);
        w16(nf);
        w16(nc);
        w16(loop_total);
        for (int i = 0; i < k; ++i) w8(rep[i]);
        for (int i = 0; i < nv_live; ++i)
            for (int t = 0; t < 3; ++t) w8(lab[vorder[i]][t]);
        uint64_t isov = 0;  // nv_live <= 64 in every variant that emits through this path
        uint8_t isovb[MV];
        for (int i = 0; i < MV; ++i) isovb[i] = 0;
        int niso = 0, nloop = 0, nbnd = 0;
        for (int i = 0; i < nf; ++i) {
            int f = forder[i];
            w8(fsupp[f]);
            w8(fneg[f] == kNoCell ? 1 : 0);
            w16(cnew[fpos[f]]);
            w16(fneg[f] == kNoCell ? 0xFFFF : cnew[fneg[f]]);
            w16(flen[f]);
            if (plane_is_iso(fsupp[f])) {
                ++niso;
                nloop += flen[f];
                if (fneg[f] == kNoCell) ++nbnd;
                for (int j = 0; j < flen[f]; ++j) isovb[vnew[loops[cur][foff[f] + j]]] = 1;
            }
        }
        (void)isov;
        for (int i = 0; i < nf; ++i) {
            int f = forder[i];
            int L = flen[f];
            int jm = 0;
            for (int j = 1; j < L; ++j)
                if (vnew[loops[cur][foff[f] + j]] < vnew[loops[cur][foff[f] + jm]]) jm = j;
            for (int t = 0; t < L; ++t) w16(vnew[loops[cur][foff[f] + (jm + t) % L]]);
        }
        for (int i = 0; i < nc; ++i) {
            uint64_t s = csign[corder[i]];
            for (int b = 0; b < 8; ++b) w8((int)((s >> (8 * b)) & 0xFF));
        }
        int nisov = 0;
        for (int i = 0; i < nv_live; ++i) nisov += isovb[i];
        sum.n_iso_v = (uint16_t)nisov;
        sum.n_iso_f = (uint16_t)niso;
        sum.n_iso_loop = (uint16_t)nloop;
        sum.n_bnd_f = (uint16_t)nbnd;
    }
};

}  // namespace ria
