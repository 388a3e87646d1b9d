// Trie node of the generated polynomial tables (csrc/gen/poly*_tables.inc).
#pragma once

namespace mbpol {

// Interior node: coefficient (FP32 hi/lo pair), variable, index one past its
// last child in the next level.  Leaf: coefficient, variable, 0.
struct PolyNode {
    float hi, lo;
    int var, end;
};

}  // namespace mbpol
