// iso_reps.cpp -- representative isovalue selection on the host.
//
// Bruckner & Moeller's scheme as the reference implements it
// (types/src/SimilarityMap.cpp:88-227):
//  * prioritize: over a contiguous run of map rows, the row with the highest
//    mean similarity to the run (first maximum wins) gets priority
//    size * mean; the run is split at that row and both halves recurse;
//  * selection: repeatedly take the highest priority (ties: lower map row,
//    where the reference's Fibonacci heap leaves the order unspecified) and
//    divide every remaining priority by (1 + similarity to the pick).  Like the
//    reference, the remaining entries take over the pick's isovalue field.
// All arithmetic is FP32 in the reference's order.
#include <cstring>
#include <vector>

#include "isosim.h"

namespace {

struct Rep {
    float isovalue, priority;
    int id, map_id;
};

void prioritize(const float *ism, int m, const std::vector<Rep> &elems, std::vector<Rep> &heap)
{
    if (elems.empty()) return;
    const int ne = (int)elems.size();
    std::vector<float> mean(ne);
    for (int i = 0; i < ne; ++i) {
        float sum = 0.0f;
        for (int j = 0; j < ne; ++j) sum += ism[(size_t)elems[i].map_id * m + elems[j].map_id];
        mean[i] = sum / (float)ne;
    }
    float best = -1.0f;
    int cur = -1;
    for (int i = 0; i < ne; ++i)
        if (mean[i] > best) {
            best = mean[i];
            cur = i;
        }
    if (cur < 0) cur = 0;  // all means NaN: take the first row
    const Rep c = elems[cur];
    heap.push_back(Rep{c.isovalue, (float)ne * mean[cur], c.id, c.map_id});
    std::vector<Rep> smaller, bigger;
    for (int i = 0; i < ne; ++i) {
        if (elems[i].map_id < c.map_id) smaller.push_back(elems[i]);
        else if (i != cur) bigger.push_back(elems[i]);
    }
    prioritize(ism, m, smaller, heap);
    prioritize(ism, m, bigger, heap);
}

}  // namespace

extern "C" int iso_select_representatives(const float *ism, int m, const int32_t *ids, const float *isovalues, int cnt,
                                          iso_rep *out)
{
    if (!ism || !ids || !isovalues || !out || m < 0 || cnt < 0) return ISO_ERR_ARG;
    std::vector<Rep> elems(m), heap;
    for (int i = 0; i < m; ++i) elems[i] = Rep{isovalues[ids[i]], -1.0f, ids[i], i};
    heap.reserve(m);
    prioritize(ism, m, elems, heap);
    int taken = 0;
    while (taken < cnt && !heap.empty()) {
        size_t top = 0;
        for (size_t h = 1; h < heap.size(); ++h)
            if (heap[h].priority > heap[top].priority ||
                (heap[h].priority == heap[top].priority && heap[h].map_id < heap[top].map_id))
                top = h;
        const Rep e = heap[top];
        out[taken++] = iso_rep{e.isovalue, e.priority, e.id, e.map_id};
        for (size_t h = 0; h < heap.size(); ++h) {
            if (h == top) continue;
            float p = heap[h].priority;
            p /= (1.0f + ism[(size_t)e.map_id * m + heap[h].map_id]);
            heap[h].priority = p;
            heap[h].isovalue = e.isovalue;
        }
        heap.erase(heap.begin() + (long)top);
    }
    return taken;
}
