// The binary heap of a std::priority_queue<int, std::vector<int>, Cmp>, host
// and device: the same element comes out on top after the same pushes and
// pops, ties included, as with the GNU C++ library's heap algorithms (hole
// based: a push moves the new element up from the end; a pop moves the last
// element into the root's place by sliding the hole down to a leaf, always
// toward the higher-priority child, then moving the element up).  The active
// layers' event queue (src/ActiveLayers.h, PenaltyGroupComparator) fires
// groups in this order, so their order decides every result.
//
// Elements are group ids; `lower(a, b)` is the comparator: true when a has
// lower priority than b.
#pragma once

#include "ccd_common.h"

namespace ccd {

template <class Lower>
CCD_HDI void heap_sift_up(int *heap, int hole, int top, int value, Lower lower) {
  int parent = (hole - 1) / 2;
  while (hole > top && lower(heap[parent], value)) {
    heap[hole] = heap[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  heap[hole] = value;
}

// priority_queue::push: append, then sift up.  *size grows by one.
template <class Lower>
CCD_HDI void heap_push(int *heap, int *size, int value, Lower lower) {
  const int hole = (*size)++;
  heap_sift_up(heap, hole, 0, value, lower);
}

// priority_queue::pop: the top leaves; *size shrinks by one.
template <class Lower>
CCD_HDI void heap_pop(int *heap, int *size, Lower lower) {
  const int len = *size - 1;  // elements left
  if (len > 0) {
    const int value = heap[len];
    heap[len] = heap[0];
    int hole = 0, child = 0;
    while (child < (len - 1) / 2) {
      child = 2 * (child + 1);
      if (lower(heap[child], heap[child - 1])) child--;
      heap[hole] = heap[child];
      hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
      child = 2 * (child + 1);
      heap[hole] = heap[child - 1];
      hole = child - 1;
    }
    heap_sift_up(heap, hole, 0, value, lower);
  }
  *size = len;
}

}  // namespace ccd
