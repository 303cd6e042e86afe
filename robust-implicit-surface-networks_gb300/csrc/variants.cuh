// Capacities of the per-tet cut variants.
//   fast: one thread per tet, state in local memory, filter-only predicates; a tet that needs an
//         exact predicate or more room is deferred.
//   big:  one tet per block with its state in shared memory, exact predicates, the full range of the
//         8-bit vertex and cell ids (about 13 planes in general position).
#pragma once
#include "cut_ia_warp.cuh"
#include "cut_mi.cuh"
#include "cut_mi_merge.cuh"

namespace ria {
using IACutFast = IACut<32, 48, 16, 192, false>;
// exact variants: the full range of the 8-bit vertex and cell ids (255 vertices, 254 cells); one tet
// per block with the state in shared memory (about 44 KB / 31 KB)
using IACutBig = IACut<255, 1024, 254, 8192, true>;
using MICutFast = MICut<32, 24, 160, 48, 48, 256, false>;
// mid-size filtered variants for the heavy bins (four or more active functions): one thread per tet,
// state in local memory, about four times the fast capacity
using IACutMid = IACut<128, 256, 64, 1024, false>;
using MICutMid = MICut<96, 96, 640, 128, 128, 1024, false>;
using MICutBig = MICut<255, 255, 2048, 255, 512, 4096, true>;
// warp variant: one warp per tet, state in shared memory, exact predicates (32 cells)
using IAWarpCutDev = IAWarpCut<64, 128, 640>;
// the same for the light bins' leftovers (three to five distinct planes): three quarters of the
// vertex, face and loop room (7 KB against 9 KB, 7 resident blocks per SM against 6); a tet that
// does not fit goes to IAWarpCutDev.  On the large degenerate workload this size measured fastest:
// the half-size state (9 blocks) sent more tets to the second launch, whose few long cuts run after
// the first launch ends
using IAWarpCutLight = IAWarpCut<48, 96, 480>;
}  // namespace ria
