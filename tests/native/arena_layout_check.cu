// Host-only check of the per-sequence arena layouts (no GPU needed): every
// region lies inside the arena, regions do not overlap, FP64 regions are
// 8-byte aligned, and every region is large enough for what the kernels
// index into it.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <algorithm>

#include "../../contrafold_gpu_gb300/csrc/cf_device.cuh"

using namespace cf;

struct Reg { const char* name; int64_t lo, hi; };   // [lo, hi) in 4-byte words

static int check(const char* what, int L, std::vector<Reg> r, int64_t total) {
    std::sort(r.begin(), r.end(), [](const Reg& a, const Reg& b) { return a.lo < b.lo; });
    for (size_t k = 0; k < r.size(); ++k) {
        if (r[k].lo < 0 || r[k].hi > total || r[k].hi < r[k].lo) {
            std::printf("%s L=%d: region %s [%lld,%lld) outside arena of %lld words\n", what, L, r[k].name,
                        (long long)r[k].lo, (long long)r[k].hi, (long long)total);
            return 1;
        }
        if (k && r[k].lo < r[k - 1].hi) {
            std::printf("%s L=%d: %s overlaps %s\n", what, L, r[k].name, r[k - 1].name);
            return 1;
        }
    }
    return 0;
}

int main() {
    int bad = 0;
    const int Ls[] = {0, 1, 2, 3, 30, 31, 32, 33, 127, 128, 200, 399, 1000, 4097, 32767};
    for (int L : Ls) {
        const int64_t tri = tri_size(L);
        const Arena32 a = arena32(L);
        // FCo .. FM2o hold tri cells; F5/F5o/up hold L+2; FB two buffers of L+2;
        // pair list: poff L+2 ints + tri int16; MEA queue 4L+8 ints.
        bad |= check("arena32", L, {
            {"FC", a.FC, a.FC + tri}, {"FM", a.FM, a.FM + tri}, {"FM1", a.FM1, a.FM1 + tri},
            {"F5", a.F5, a.F5 + L + 2}, {"FB", a.FB, a.FB + 2 * pad32(L + 2)},
            {"PL", a.PL, a.PL + (L + 3) + (tri + 1) / 2},
            {"FCo", a.FCo, a.FCo + tri}, {"FMo", a.FMo, a.FMo + tri}, {"FM1o", a.FM1o, a.FM1o + tri},
            {"FM2o", a.FM2o, a.FM2o + tri}, {"F5o", a.F5o, a.F5o + L + 2}, {"up", a.up, a.up + L + 2},
            {"queue", a.queue, a.queue + 4 * (int64_t)L + 8}}, a.total);
        if (a.FB + 2 * pad32(L + 2) > a.PL) { std::printf("FB spills into PL\n"); bad = 1; }
        if (arena32_inside_words(L) != a.FCo) { std::printf("inside prefix mismatch L=%d\n", L); bad = 1; }
        const Arena64 b = arena64(L);
        // doubles -> words: x2
        bad |= check("arena64", L, {
            {"FC", 2 * b.FC, 2 * (b.FC + tri)}, {"FM", 2 * b.FM, 2 * (b.FM + tri)},
            {"FM1", 2 * b.FM1, 2 * (b.FM1 + tri)}, {"F5", 2 * b.F5, 2 * (b.F5 + L + 2)},
            {"FB", 2 * b.FB, 2 * (b.FB + 2 * pad32(L + 2))},
            {"PL", b.PL, b.PL + (L + 3) + (tri + 1) / 2},
            {"stack", b.stack, b.stack + 3 * (4 * (int64_t)L + 16)}}, b.total);
        if (b.total % 2 || b.PL % 2) { std::printf("arena64 misaligned L=%d\n", L); bad = 1; }
        if (a.total % 32 || b.total % 32) { std::printf("arena not 128-byte padded L=%d\n", L); bad = 1; }
    }
    std::printf(bad ? "FAIL\n" : "OK\n");
    return bad;
}
