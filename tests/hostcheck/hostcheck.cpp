// Test-only harness: compiles the device per-tet cut headers for the host so that their logic can be
// checked against the CPU oracle without a GPU.  Never linked into the product library.
#include <cstring>
#include <vector>

#include "../../robust-implicit-surface-networks_gb300/csrc/cut_mi.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/cut_mi_warp.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/variants.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/lookup2.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/cut_ia_warp.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/sqrt_rn.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/div_rn.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/robust.cuh"

using namespace ria;

template <class C, class S>
static int finish(C* c, int st, uint8_t* buf, int cap, uint16_t* summary) {
    if (st != CUT_OK) return -10 - st;
    c->canonicalize();
    int n = c->record_size();
    if (n > cap) return -3;
    S s;
    c->emit(buf, s);
    std::memcpy(summary, &s, sizeof(S));
    return n;
}

// one tet through a warp variant's state (one lane: its lane-parallel loops run serially)
template <class W>
int warp_cut(int k, const double* planes, uint8_t* buf, int cap, uint16_t* summary) {
    if (k > kWarpMaxK) return -11;
    auto* c = new W();
    for (int i = 0; i < 4 * k; ++i) c->pl[i] = planes[i];
    Lanes L;
    int st = c->run(L, k);
    int r = 0;
    if (st != CUT_OK) {
        r = -10 - st;
    } else {
        c->canonicalize(L);
        r = c->record_size();
        if (r > cap) {
            r = -3;
        } else {
            IASummary s;
            c->emit(L, buf, s);
            std::memcpy(summary, &s, sizeof(s));
        }
    }
    delete c;
    return r;
}

// big: 0 the small filtered variant, 1 the exact variant, 2 the mid-size filtered variant, 3 the
// warp variant, 4 the warp variant's light state (one lane: its lane-parallel loops run serially)
extern "C" int hc_ia_cut(int k, const double* planes, int big, uint8_t* buf, int cap, uint16_t* summary) {
    if (big == 4) return warp_cut<IAWarpCutLight>(k, planes, buf, cap, summary);
    if (big == 3) {
        if (k > kWarpMaxK) return -11;
        auto* c = new IAWarpCutDev();
        for (int i = 0; i < 4 * k; ++i) c->pl[i] = planes[i];
        Lanes L;
        int st = c->run(L, k);
        int r = 0;
        if (st != CUT_OK) {
            r = -10 - st;
        } else {
            c->canonicalize(L);
            r = c->record_size();
            if (r > cap) {
                r = -3;
            } else {
                IASummary s;
                c->emit(L, buf, s);
                std::memcpy(summary, &s, sizeof(s));
            }
        }
        delete c;
        return r;
    }
    if (big == 2) {
        auto* c = new IACutMid();
        int r = finish<IACutMid, IASummary>(c, c->run(planes, k), buf, cap, summary);
        delete c;
        return r;
    }
    if (big) {
        auto* c = new IACutBig();
        int r = finish<IACutBig, IASummary>(c, c->run(planes, k), buf, cap, summary);
        delete c;
        return r;
    }
    auto* c = new IACutFast();
    int r = finish<IACutFast, IASummary>(c, c->run(planes, k), buf, cap, summary);
    delete c;
    return r;
}

// big == 3: the split path of the device (the per-tet preparation and one warp clipper per material,
// then the lane-parallel merge, each with one lane)
static int mi_split(int k, const double* mats, uint8_t* buf, int cap, uint16_t* summary) {
    using SplitClip = MIWarpClip<32, 32, 192>;  // the device's warp clipper
    using SplitCell = MICell<32, 32, 192>;
    if (k > 32) return -11;
    std::vector<SplitCell> cells(k);
    uint8_t has[32] = {};
    Lanes L1;
    auto* prep = new MIPrep();
    mi_prepare_lanes(L1, mats, k, *prep);
    auto* c = new MICut<32, 32, 192, 1, 1, 1, false>();  // the serial preparation, to compare with
    int st = c->prepare(mats, k);
    for (int i = 0; i < k && st == CUT_OK; ++i)
        if (prep->rep[i] != c->rep[i]) st = CUT_FAIL;
    auto* cm = new SplitClip();
    for (int m = 0; m < k && st == CUT_OK; ++m) {
        if (prep->has_cell(4 + m) != c->has_cell(4 + m)) {
            st = CUT_FAIL;  // the two preparations disagree
            break;
        }
        if (!prep->has_cell(4 + m)) continue;
        bool empty = false;
        st = cm->clip(L1, mats, k, *prep, 4 + m, empty);
        if (st == CUT_OK && !empty) {
            st = cm->export_cell(L1, cells[m]);
            has[m] = 1;
        }
    }
    delete cm;
    int r = -10 - st;
    if (st == CUT_OK) {
        auto* mg = new MIMerge<SplitCell>();
        Lanes L;
        st = mg->run(L, cells.data(), has, k);
        if (st != CUT_OK) {
            r = -10 - st;
        } else {
            r = mg->record_size(k);
            if (r > cap) {
                r = -3;
            } else {
                MISummary s;
                mg->emit(L, cells.data(), k, prep->rep, buf, s);
                std::memcpy(summary, &s, sizeof(s));
            }
        }
        delete mg;
    }
    delete c;
    delete prep;
    return r;
}

extern "C" int hc_mi_cut(int k, const double* mats, int big, uint8_t* buf, int cap, uint16_t* summary) {
    if (big == 3) return mi_split(k, mats, buf, cap, summary);
    if (big == 2) {
        auto* c = new MICutMid();
        int r = finish<MICutMid, MISummary>(c, c->run(mats, k), buf, cap, summary);
        delete c;
        return r;
    }
    if (big) {
        auto* c = new MICutBig();
        int r = finish<MICutBig, MISummary>(c, c->run(mats, k), buf, cap, summary);
        delete c;
        return r;
    }
    auto* c = new MICutFast();
    int r = finish<MICutFast, MISummary>(c, c->run(mats, k), buf, cap, summary);
    delete c;
    return r;
}

extern "C" int hc_det_sign(const double* M, int n) { return det_sign_exact(M, n); }

// secondary lookup keys: returns 1 and the key, or 0 when no key is formed
extern "C" int hc_ia_key2(const double* rows, uint32_t* key) { return ia_key2(rows, *key) ? 1 : 0; }
extern "C" int hc_mi_key3(const double* rows, uint32_t* key) { return mi_key3(rows, *key) ? 1 : 0; }
extern "C" int hc_ia_key3(const double* rows, uint64_t* key) { return ia_key3(rows, *key) ? 1 : 0; }

// The one-effective-plane path of the fast kernel: the one-plane table is built by the exact variant
// from corner values in {-1, 0, 1}, as on the device.
extern "C" int hc_ia_template(int k, const double* planes, uint8_t* buf, int cap, uint16_t* summary) {
    static uint8_t table[81][256];
    static bool built = false;
    if (!built) {
        for (int p = 0; p < 81; ++p) {
            double pl[4];
            int q = p;
            for (int c = 0; c < 4; ++c) {
                pl[c] = (double)(q % 3) - 1.0;
                q /= 3;
            }
            auto* c = new IACutBig();
            c->run(pl, 1);
            c->canonicalize();
            IASummary s;
            c->emit(table[p], s);
            delete c;
        }
        built = true;
    }
    uint8_t rep[64];
    int first;
    int eff = ia_group_planes(planes, k, rep, first);
    if (eff > 1) return -1;
    const uint8_t* tmpl = table[eff ? ia_sign_pattern(planes + 4 * first) : 80];
    int n = ia_template_record_size(tmpl, k);
    if (n > cap) return -3;
    ia_record_from_template(tmpl, k, rep, eff, first, buf);
    IASummary s, st;
    ia_record_summary(buf, s);
    ia_record_summary(tmpl, st, rep, k);  // the device's summary, from the template
    if (std::memcmp(&s, &st, sizeof(s)) != 0) return -99;
    {  // the device's word-wise writer
        uint64_t words[512] = {};
        WordSink o{words};
        ia_template_relabel1(tmpl, k, rep, eff, first, o);
        if (n > (int)sizeof(words) || std::memcmp(words, buf, n) != 0) return -98;
    }
    std::memcpy(summary, &s, sizeof(s));
    return n;
}

// The two-group path of the fast kernel: the two representative planes cut alone (k = 2), their
// record relabelled for the tet, as on a secondary-lookup hit or miss.
extern "C" int hc_ia_template2(int k, const double* planes, uint8_t* buf, int cap, uint16_t* summary) {
    uint8_t rep[64];
    int first;
    if (ia_group_planes(planes, k, rep, first) != 2) return -1;
    int r[2], n = 0;
    for (int i = 0; i < k; ++i)
        if (rep[i] == 4 + i) {
            if (n == 2) return -2;
            r[n++] = i;
        }
    if (n != 2) return -2;
    double two[8];
    for (int c = 0; c < 4; ++c) {
        two[c] = planes[4 * r[0] + c];
        two[4 + c] = planes[4 * r[1] + c];
    }
    static uint8_t rec2[1024];
    uint16_t s2[16];
    const int size2 = hc_ia_cut(2, two, 0, rec2, sizeof(rec2), s2);
    if (size2 < 0) return size2;
    const int size = ia_template_record_size(rec2, k);
    if (size > cap) return -3;
    ia_record_from_template2(rec2, k, rep, r[0], r[1], buf);
    IASummary s, st;
    ia_record_summary(buf, s);
    ia_record_summary(rec2, st, rep, k);  // the device's summary, from the template
    if (std::memcmp(&s, &st, sizeof(s)) != 0) return -99;
    {  // the device's word-wise writer
        uint64_t words[512] = {};
        WordSink o{words};
        ia_template_relabel2(rec2, k, rep, r[0], r[1], o);
        if (size > (int)sizeof(words) || std::memcmp(words, buf, size) != 0) return -98;
    }
    std::memcpy(summary, &s, sizeof(s));
    return size;
}

extern "C" int hc_sizes(int* out) {
    out[0] = (int)sizeof(IACutFast);
    out[1] = (int)sizeof(IACutBig);
    out[2] = (int)sizeof(MICutFast);
    out[3] = (int)sizeof(MICutBig);
    return 0;
}

// the sampler's square root; perturb != 0 moves its seed by perturb * 2^-20 (relative), beyond the
// FP32 estimate's error, to show the margin of the two Newton steps
extern "C" void hc_sqrt_rn(const double* in, double* out, int64_t n, int perturb) {
    for (int64_t i = 0; i < n; ++i) {
        uint64_t x;
        int e;
        if (perturb == 0 || !sqrt_split(in[i], x, e)) {
            out[i] = sqrt_rn(in[i]);
            continue;
        }
        const uint64_t r0 = sqrt_seed(x);
        out[i] = sqrt_rn_finish(x, e, (uint64_t)((int64_t)r0 + perturb * (int64_t)(r0 >> 20)));
    }
}

// the vertex emission's division (div_rn.cuh)
extern "C" void hc_div_rn(const double* a, const double* b, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = div_rn(a[i], b[i]);
}

// ---- robust test (robust.cuh): the device's per-tet classification with a cut wrapper that can forge
// a failure of the first or second cut, or a different face count of the second, so that the test can
// check that every outcome is reported.  forge: 0 none, 1 count mismatch, 2 first cut fails, 3 second
// cut fails.
namespace ria {
template <class Base>
struct ForgeCut : Base {
    int forge = 0, calls = 0;
    int run(const double* rows, int k) {
        ++calls;
        if ((forge == 2 && calls == 1) || (forge == 3 && calls == 2)) return CUT_FAIL;
        return Base::run(rows, k);
    }
};
template <class Base>
void cut_counts(const ForgeCut<Base>& c, int out[3]) {
    cut_counts(static_cast<const Base&>(c), out);
    if (c.forge == 1 && c.calls == 2) out[1] += 1;
}
}  // namespace ria

extern "C" int hc_robust(int mi, int k, const double* rows, int forge) {
    std::vector<double> buf(8 * (size_t)(k > 0 ? k : 1));
    for (int i = 0; i < 4 * k; ++i) buf[i] = rows[i];
    int r;
    if (mi) {
        auto* c = new ForgeCut<MICutBig>();
        c->forge = forge;
        r = robust_tet(*c, buf.data(), k);
        delete c;
    } else {
        auto* c = new ForgeCut<IACutBig>();
        c->forge = forge;
        r = robust_tet(*c, buf.data(), k);
        delete c;
    }
    return r;
}
