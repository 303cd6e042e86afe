// Test-only harness: compiles the device per-tet cut headers for the host so that their logic can be
// checked against the CPU oracle without a GPU.  Never linked into the product library.
#include <cstring>

#include "../../robust-implicit-surface-networks_gb300/csrc/cut_mi.cuh"
#include "../../robust-implicit-surface-networks_gb300/csrc/variants.cuh"

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

extern "C" int hc_ia_cut(int k, const double* planes, int big, uint8_t* buf, int cap, uint16_t* summary) {
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

extern "C" int hc_mi_cut(int k, const double* mats, int big, uint8_t* buf, int cap, uint16_t* summary) {
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
