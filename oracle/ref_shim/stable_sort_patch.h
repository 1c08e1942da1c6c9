// Forced-include header for the reference checker build (oracle/Makefile.ref).
//
// HeavyRT sorts (Morton code, triangle id) pairs with std::sort on the code
// alone (core/builders/lbvh.cpp:755), so the order among equal codes is left
// to the standard library.  The checker pins it to the stable order
// (tie-break = original triangle index), which is what the engine's LSD radix
// sort and the C restatement produce.  This overload is more specialised than
// the library template, so overload resolution picks it for that one call.
#pragma once
#include <algorithm>
#include <vector>
#include "LiteMath.h"

namespace std
{
  template <class Cmp>
  inline void sort(std::vector<LiteMath::uint2>::iterator first, std::vector<LiteMath::uint2>::iterator last, Cmp cmp)
  {
    std::stable_sort(first, last, cmp);
  }
}
