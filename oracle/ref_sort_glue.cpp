/*
 * C entry point around the reference's own preorder_by_x (Tools.cpp:46-66),
 * compiled from the reference sources by oracle/build_ref.py.  TEST
 * INFRASTRUCTURE ONLY: it pins the per-module x-sort permutation (including
 * the order of equal-x hits) of the oracle and of the product's sort.
 */
#include <cstdint>
#include <cstring>
#include <vector>

void preorder_by_x(std::vector<const std::vector<uint8_t>*>& input);   // Tools.h:47

extern "C" int ref_preorder_by_x(uint8_t* const* blobs, const uint64_t* sizes, int n) {
  if (n <= 0) return 0;
  std::vector<std::vector<uint8_t>> store(n);
  std::vector<const std::vector<uint8_t>*> ptrs(n);
  for (int i = 0; i < n; ++i) {
    store[i].assign(blobs[i], blobs[i] + sizes[i]);
    ptrs[i] = &store[i];
  }
  preorder_by_x(ptrs);   // sorts in place through the const pointers, as the reference does
  for (int i = 0; i < n; ++i) std::memcpy(blobs[i], store[i].data(), sizes[i]);
  return 0;
}
