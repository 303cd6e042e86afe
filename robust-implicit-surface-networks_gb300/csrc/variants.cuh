// Capacities of the per-tet cut variants.
//   fast: one thread per tet, state in local memory, filter-only predicates; a tet that needs an
//         exact predicate or more room is deferred.
//   big:  state in global scratch, exact predicates, room for up to ~10 active functions.
#pragma once
#include "cut_mi.cuh"

namespace ria {
using IACutFast = IACut<32, 48, 16, 192, false>;
using IACutBig = IACut<128, 256, 64, 1024, true>;
using MICutFast = MICut<32, 24, 160, 48, 48, 256, false>;
using MICutBig = MICut<96, 96, 640, 128, 128, 1024, true>;
}  // namespace ria
