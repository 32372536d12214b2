// batch_order.h -- the batch plans' work-list order (host only, no CUDA
// headers; batch.cpp instantiates it, tests/cpp/test_batch_order.cpp checks
// its invariants).
#pragma once
#include <cstddef>
#include <deque>
#include <vector>

namespace glsfft {

// Item order: pass 0 of the images in order; pass p+1 of an image enters the
// list once `lag` items have been listed after its pass p (the work resident
// blocks are busy with in the meantime), so its inputs are fresh in L2 and
// rarely still being written.  An item of pass p+1 carries `need` = the tile
// count of pass p, whose tiles all precede it in the list -- blocks claim
// items in list order, so every wait is for items already claimed and the
// launch cannot deadlock.  Image: row_tiles, col_tiles; Pass: along_rows;
// Item: {image, pass, tile, need}.
template <class Item, class Image, class Pass>
std::vector<Item> order_work(const std::vector<Image> &ims, const std::vector<Pass> &passes,
                             int lag) {
    struct Pending {
        size_t ready_at;
        int image, pass, need;
    };
    std::vector<Item> out;
    std::deque<Pending> pend;  // ready_at is non-decreasing in push order
    auto tiles = [&](int i, int p) {
        return passes[p].along_rows ? ims[i].row_tiles : ims[i].col_tiles;
    };
    auto emit = [&](int i, int p, int need) {
        const int n = tiles(i, p);
        for (int t = 0; t < n; t++) out.push_back(Item{i, p, t, need});
        if (p + 1 < (int)passes.size())
            pend.push_back(Pending{out.size() + (size_t)lag, i, p + 1, n});
    };
    for (int i = 0; i < (int)ims.size(); i++) {
        while (!pend.empty() && pend.front().ready_at <= out.size()) {
            Pending q = pend.front();
            pend.pop_front();
            emit(q.image, q.pass, q.need);
        }
        emit(i, 0, 0);
    }
    while (!pend.empty()) {
        Pending q = pend.front();
        pend.pop_front();
        emit(q.image, q.pass, q.need);
    }
    return out;
}

}  // namespace glsfft
