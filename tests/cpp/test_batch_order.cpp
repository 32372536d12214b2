// Host unit test of the batch plans' work-list order
// (glscv_gb300/csrc/batch_order.h), compiled without CUDA: every
// (image, pass, tile) is listed exactly once, and every item of a later pass
// follows all tiles of its image's previous pass and waits for exactly that
// many -- blocks claim items in list order, so no wait can be for an item
// that no block has claimed.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <tuple>
#include <vector>

#include "batch_order.h"

struct Im {
    int row_tiles, col_tiles;
};
struct Ps {
    int along_rows;
};
struct It {
    int image, pass, tile, need;
};

static int failures = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);        \
            if (++failures > 20) std::exit(1);                     \
        }                                                          \
    } while (0)

int main() {
    std::mt19937 rng(12345);
    for (int trial = 0; trial < 400; trial++) {
        const int n_images = 1 + (int)(rng() % 40);
        const int n_passes = (rng() % 2) ? 4 : 2;
        std::vector<Im> ims(n_images);
        for (auto &im : ims) im = {1 + (int)(rng() % 300), 1 + (int)(rng() % 300)};
        std::vector<Ps> ps;
        for (int p = 0; p < n_passes; p++) ps.push_back({p % 2 == 0 ? 1 : 0});
        const int lag = (int)(rng() % 3000);
        const std::vector<It> items = glsfft::order_work<It>(ims, ps, lag);
        auto tiles = [&](int i, int p) { return ps[p].along_rows ? ims[i].row_tiles : ims[i].col_tiles; };
        size_t total = 0;
        for (int i = 0; i < n_images; i++)
            for (int p = 0; p < n_passes; p++) total += tiles(i, p);
        CHECK(items.size() == total);
        std::map<std::tuple<int, int, int>, int> seen;
        std::vector<std::vector<int>> listed(n_images, std::vector<int>(n_passes, 0));
        int last_image0 = -1;
        for (const It &it : items) {
            CHECK(it.image >= 0 && it.image < n_images && it.pass >= 0 && it.pass < n_passes);
            CHECK(it.tile >= 0 && it.tile < tiles(it.image, it.pass));
            const int count = ++seen[std::make_tuple(it.image, it.pass, it.tile)];
            CHECK(count == 1);
            if (it.pass == 0) {
                CHECK(it.need == 0);
                CHECK(it.image >= last_image0);  // pass 0 in image order
                last_image0 = it.image;
            } else {
                CHECK(it.need == tiles(it.image, it.pass - 1));
                CHECK(listed[it.image][it.pass - 1] == it.need);  // all of them already listed
            }
            listed[it.image][it.pass]++;
        }
    }
    if (failures) return 1;
    std::printf("ALL OK\n");
    return 0;
}
