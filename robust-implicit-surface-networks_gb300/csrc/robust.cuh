// The reference's robustness test of one tet (src/implicit_arrangement.cpp:137-243 and
// src/material_interface.cpp:174-287): the tet is cut with its rows in the given order and in the
// reversed order, and the outcome is classified as the reference classifies it:
//   type 2  the cut in the given order fails ("crash in the normal order");
//   type 3  the given order succeeds and the reversed order fails;
//   type 1  both succeed and the vertex, face or cell counts differ ("inconsistency").
// The exact variant reports every cut it cannot finish (an inconsistency that exact arithmetic rules
// out, an expansion overflow, or a tet beyond its capacity) as CUT_FAIL, which counts as the
// reference's crash.  A filtered variant's CUT_DEFER (undecided filter, or its smaller capacity) is
// not an outcome: it is returned as ROBUST_CAPACITY.
// Device code; also compiled for the host by the test-only harness, whose forging wrapper checks that
// every outcome is counted.
#pragma once
#include "cut_ia.cuh"
#include "cut_mi.cuh"

namespace ria {

enum : int { ROBUST_OK = 0, ROBUST_TYPE1 = 1, ROBUST_TYPE2 = 2, ROBUST_TYPE3 = 3, ROBUST_CAPACITY = 4 };

// vertex, face and cell counts of a finished, canonicalized cut
template <int MV, int MF, int MC, int ML, bool EXACT>
RIA_HDI void cut_counts(const IACut<MV, MF, MC, ML, EXACT>& c, int out[3]) {
    out[0] = c.nv_live;
    out[1] = c.nf;
    out[2] = c.nc;
}
template <int PV, int PF, int PL, int OV, int OF, int OL, bool EXACT>
RIA_HDI void cut_counts(const MICut<PV, PF, PL, OV, OF, OL, EXACT>& c, int out[3]) {
    out[0] = c.onv;
    out[1] = c.onf;
    out[2] = c.onc;
}

// rows: room for 8k values; rows[0, 4k) hold the tet's k rows in the given order, and the reversed
// order is written to rows[4k, 8k).
template <class Cut>
RIA_HDI int robust_tet(Cut& cut, double* rows, int k) {
    for (int r = 0; r < k; ++r)
        for (int c = 0; c < 4; ++c) rows[4 * (2 * k - 1 - r) + c] = rows[4 * r + c];
    int counts[2][3];
    for (int pass = 0; pass < 2; ++pass) {
        const int st = cut.run(rows + (pass ? 4 * k : 0), k);
        if (st == CUT_DEFER) return ROBUST_CAPACITY;
        if (st != CUT_OK) return pass ? ROBUST_TYPE3 : ROBUST_TYPE2;
        cut.canonicalize();
        cut_counts(cut, counts[pass]);
    }
    if (counts[0][0] != counts[1][0] || counts[0][1] != counts[1][1] || counts[0][2] != counts[1][2])
        return ROBUST_TYPE1;
    return ROBUST_OK;
}

}  // namespace ria
