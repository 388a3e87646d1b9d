// Host check of the polynomial walks' trie split (poly_df.cu, make_split):
// every level-2 node is walked by exactly one part, every level-1 node's
// coefficient is counted exactly once, and each part's level-3 start is the
// first child of its first level-2 node.  Built by tests/test_walk_split.py
// with nvcc for each part count; no GPU is used.
#include <algorithm>
#include <cstdio>

#include "poly_df.cu"

namespace mbpol {
void count_launch() {}
namespace {
int check(const WalkSplit& s, const PolyNode* l1, int n1, const PolyNode* l2, int n2, const char* name) {
    std::vector<int> cov2(n2, 0), coef1(n1, 0);
    for (int k = 0; k < kParts; ++k) {
        const WalkPart& W = s.part[k];
        if (W.c2_0 >= W.c2_1) {
            printf("%s: part %d is empty\n", name, k);
            return 1;
        }
        int c2 = W.c2_0;
        for (int a = W.a0; a < W.a1; ++a) {
            if (!(a == W.a0 && W.skip_coef)) coef1[a]++;
            const int e2 = std::min((int)l1[a].end, W.c2_1);
            for (; c2 < e2; ++c2) cov2[c2]++;
        }
        if (c2 != W.c2_1) {
            printf("%s: part %d stops at level-2 node %d, not %d\n", name, k, c2, W.c2_1);
            return 1;
        }
        if (W.c3_0 != (W.c2_0 == 0 ? 0 : (int)l2[W.c2_0 - 1].end)) {
            printf("%s: part %d level-3 start\n", name, k);
            return 1;
        }
    }
    for (int j = 0; j < n2; ++j)
        if (cov2[j] != 1) {
            printf("%s: level-2 node %d walked %d times\n", name, j, cov2[j]);
            return 1;
        }
    for (int a = 0; a < n1; ++a)
        if (coef1[a] != 1) {
            printf("%s: level-1 coefficient %d counted %d times\n", name, a, coef1[a]);
            return 1;
        }
    printf("%s: %d parts ok\n", name, kParts);
    return 0;
}
}  // namespace
}  // namespace mbpol

int main() {
    using namespace mbpol;
    int r = check(split2(), poly2b_l1, POLY2B_N1, poly2b_l2, POLY2B_N2, "two-body");
    r |= check(split3(), poly3b_l1, POLY3B_N1, poly3b_l2, POLY3B_N2, "three-body");
    return r;
}
