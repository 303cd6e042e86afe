// CPU oracle (test infrastructure only): per-tet implicit arrangement and material interface.
//
// Restates, from the mathematics, what the reference obtains from the absent third-party
// library qnzhou/simplicial_arrangement (GIT_TAG main, unpinned):
//   compute_arrangement(std::vector<Plane<double,3>>)          called at
//       src/implicit_arrangement.cpp:279,283
//   compute_material_interface(std::vector<Material<double,3>>) called at
//       src/material_interface.cpp:323,327
// The output honours the data contract that src/extract_mesh.cpp consumes:
//   vertices[i]  = sorted plane ids (IA: 3, MI: 4); ids 0..3 are the tet faces (id b is the face
//                  opposite tet corner b), implicit plane / material j has id 4+j
//                  (src/extract_mesh.cpp:101-105, 659)
//   faces[j]     = ordered polygon, supporting plane (IA) or positive/negative material label (MI),
//                  positive/negative cell; IA boundary faces have negative_cell = None
//                  (src/extract_mesh.cpp:240)
//   unique plane / material groups (src/extract_mesh.cpp:65-90, 848-864)
// The record is put in a canonical form so that two independent implementations can be compared
// byte for byte:
//   * a vertex is labelled by the lexicographically smallest independent set of the planes
//     through it; vertices are sorted by that label tuple;
//   * IA faces are sorted by (supporting plane, sorted vertex ids), MI faces by
//     (positive label, negative label); every loop starts at its smallest vertex id and runs
//     counter-clockwise seen from the positive side;
//   * IA cells are sorted by their sign vector over the implicit planes, MI cells by material.
#pragma once
#include <array>
#include <cstdint>
#include <vector>

namespace oracle {

constexpr uint16_t kNone16 = 0xFFFF;

struct IAFaceRec {
    int supp;
    int pos, neg;  // neg = -1: tet boundary
    std::vector<int> loop;
};

struct IARecord {
    int k = 0;
    std::vector<uint8_t> rep;  // representative label of implicit plane 4+i (0xFF: zero plane)
    std::vector<std::array<uint8_t, 3>> verts;
    std::vector<IAFaceRec> faces;
    std::vector<uint64_t> cell_sign;  // per cell, bit (4+i) set on the positive side of plane 4+i
};

struct MIFaceRec {
    int pos_label, neg_label;
    std::vector<int> loop;
};

struct MIRecord {
    int k = 0;
    std::vector<uint8_t> rep;  // representative label of material 4+i
    std::vector<std::array<uint8_t, 4>> verts;
    std::vector<MIFaceRec> faces;
    std::vector<int> cell_label;
};

struct CutStats {
    long exact_calls = 0;
};

// planes: k rows of 4 corner values.  Returns false if k exceeds 60.
bool ia_cut(int k, const double* planes, IARecord& out, CutStats* st = nullptr);
bool mi_cut(int k, const double* materials, MIRecord& out, CutStats* st = nullptr);

// byte serialisation shared with the device records (see the C-ABI header)
void ia_serialize(const IARecord& r, std::vector<uint8_t>& buf);
void mi_serialize(const MIRecord& r, std::vector<uint8_t>& buf);

}  // namespace oracle
