// Stand-in for Kokkos::BinSort and Kokkos::BinOp1D as the reference's face
// ordering uses them (BinSort over the left cell of each face with
// BinOp1D(n/2, min, max) and sort_within_bins = true). Test infrastructure
// only.
//
// Behaviour restated from the published Kokkos 2.x algorithm:
//   * BinOp1D(max_bins, min, max) has max_bins + 1 bins; key k goes to bin
//     int(mul * (k - min)) with mul = max_bins / (max - min) in double.
//   * create_permute_vector() counts the keys per bin, takes the exclusive
//     prefix sum as bin offsets and places the indices bin by bin; with one
//     thread (the Serial back end, and here always) each bin receives its
//     indices in increasing index order.
//   * With sort_within_bins, each bin is then ordered by repeated bubble
//     passes over its slots that swap two neighbours whenever the comparator
//     (keys(a) < keys(b)) is false, shortening the pass by one slot each time,
//     until a pass makes no swap. Equal keys are swapped too.
// When every key is the same, Kokkos divides by zero; here all keys then go
// to bin 0.
#ifndef MINIAERO_KOKKOS_SHIM_SORT_HPP
#define MINIAERO_KOKKOS_SHIM_SORT_HPP

#include "Kokkos_Core.hpp"

namespace Kokkos {

template <class KeyViewType>
struct BinOp1D {
  typedef typename KeyViewType::non_const_value_type key_type;
  int nbins_;
  double mul_;
  key_type min_;

  BinOp1D() : nbins_(0), mul_(0.0), min_() {}
  BinOp1D(int max_bins, key_type min, key_type max)
      : nbins_(max_bins + 1), mul_(max == min ? 0.0 : 1.0 * max_bins / (max - min)), min_(min) {}

  int max_bins() const { return nbins_; }

  template <class V>
  int bin(const V& keys, int i) const {
    return static_cast<int>(mul_ * (keys(i) - min_));
  }

  template <class V>
  bool operator()(const V& keys, int a, int b) const {
    return keys(a) < keys(b);
  }
};

template <class KeyViewType, class BinSortOp, class ExecutionSpace = DefaultExecutionSpace, class SizeType = int>
class BinSort {
 public:
  typedef View<SizeType*> offset_type;

  KeyViewType keys;
  BinSortOp bin_op;
  bool sort_within_bins;
  offset_type bin_count_atomic;
  offset_type bin_offsets;
  offset_type sort_order;

  BinSort() : sort_within_bins(false) {}
  BinSort(KeyViewType keys_, BinSortOp op, bool within = false)
      : keys(keys_),
        bin_op(op),
        sort_within_bins(within),
        bin_count_atomic("BinSort::bin_count", op.max_bins()),
        bin_offsets("BinSort::bin_offsets", op.max_bins()),
        sort_order("PermutationVector", keys_.dimension_0()) {}

  void create_permute_vector() {
    const int n = static_cast<int>(keys.dimension_0());
    const int nb = bin_op.max_bins();
    std::vector<SizeType> count(static_cast<size_t>(nb), 0);
    for (int i = 0; i < n; ++i) ++count[static_cast<size_t>(bin_op.bin(keys, i))];
    SizeType acc = 0;
    for (int b = 0; b < nb; ++b) {
      bin_count_atomic(b) = count[static_cast<size_t>(b)];
      bin_offsets(b) = acc;
      acc += count[static_cast<size_t>(b)];
    }
    std::vector<SizeType> fill(static_cast<size_t>(nb), 0);
    for (int i = 0; i < n; ++i) {
      const int b = bin_op.bin(keys, i);
      sort_order(bin_offsets(b) + fill[static_cast<size_t>(b)]++) = i;
    }
    if (!sort_within_bins) return;
    for (int b = 0; b < nb; ++b) {
      const SizeType first = bin_offsets(b);
      SizeType end = first + count[static_cast<size_t>(b)];
      bool swapped = true;
      while (swapped && end - first > 1) {
        swapped = false;
        SizeType carried = sort_order(first);
        for (SizeType k = first + 1; k < end; ++k) {
          const SizeType next = sort_order(k);
          if (!bin_op(keys, carried, next)) {
            sort_order(k - 1) = next;
            sort_order(k) = carried;
            swapped = true;
          } else {
            carried = next;
          }
        }
        --end;
      }
    }
  }

  offset_type get_permute_vector() const { return sort_order; }
};

}  // namespace Kokkos

#endif
