// Host-only unit test of the serving loop's device-memory arena
// (glscv_gb300/csrc/arena.h): first fit, alignment, coalescing, refusal.
#include <cstdio>
#include <vector>

#include "arena.h"

using glsfft::Arena;

static int failures = 0;
#define EXPECT(c)                                                   \
    do {                                                            \
        if (!(c)) {                                                 \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);        \
            failures++;                                             \
        }                                                           \
    } while (0)

int main() {
    Arena a(4096);
    EXPECT(a.capacity() == 4096);
    size_t x = a.alloc(100), y = a.alloc(256), z = a.alloc(1000);
    EXPECT(x == 0 && y == 256 && z == 512);  // 256-byte alignment
    EXPECT(a.in_use() == 256 + 256 + 1024);
    EXPECT(a.alloc(4096) == Arena::kFail);
    EXPECT(!a.fits(3000) && a.fits(2560));
    EXPECT(a.release(y));
    EXPECT(!a.release(y));          // double free refused
    EXPECT(!a.release(12345));      // unknown offset refused
    EXPECT(a.alloc(200) == 256);    // first fit reuses the hole
    EXPECT(a.release(256) && a.release(x) && a.release(z));
    EXPECT(a.in_use() == 0 && a.blocks() == 0);
    EXPECT(a.largest_free() == 4096);  // everything coalesced back
    // churn: random alloc/free keeps the invariants
    std::vector<size_t> live;
    unsigned s = 1;
    for (int i = 0; i < 10000; i++) {
        s = s * 1103515245u + 12345u;
        if ((s >> 16) % 3 && live.size() < 12) {
            size_t o = a.alloc(((s >> 8) % 700) + 1);
            if (o != Arena::kFail) live.push_back(o);
        } else if (!live.empty()) {
            const size_t k = (s >> 4) % live.size();
            EXPECT(a.release(live[k]));
            live.erase(live.begin() + k);
        }
        EXPECT(a.in_use() <= a.capacity());
    }
    for (size_t o : live) EXPECT(a.release(o));
    EXPECT(a.in_use() == 0 && a.largest_free() == 4096);
    if (failures) {
        std::printf("%d FAILURES\n", failures);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
