/* Stand-in for the reference's vendored CUB (include/cub, ~2015 v1.x), which does not compile
 * with current CUDA.  Test infrastructure only.  The reference calls one function,
 * cub::DeviceRadixSort::SortPairs (kernel/SortReorder.h:39-47, sizing call :221-238).  CUB
 * documents it as a stable LSD radix sort of (key, value) pairs over bits [begin_bit, end_bit):
 * restated here as a stable counting sort, 8 bits per pass. */
#pragma once
#include <cstddef>
#include <cstring>
#include <vector>

namespace cub {
struct DeviceRadixSort {
    template <class K, class V>
    static int SortPairs(void* temp, size_t& temp_bytes, const K* keys_in, K* keys_out, const V* vals_in,
                         V* vals_out, int n, int begin_bit = 0, int end_bit = (int)sizeof(K) * 8) {
        if (!temp) { temp_bytes = 16; return 0; }   // sizing call
        std::vector<K> ka(keys_in, keys_in + n), kb(n);
        std::vector<V> va(vals_in, vals_in + n), vb(n);
        for (int sh = begin_bit; sh < end_bit; sh += 8) {
            size_t cnt[257] = {0};
            for (int i = 0; i < n; ++i) cnt[((ka[i] >> sh) & 255u) + 1]++;
            for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
            for (int i = 0; i < n; ++i) {
                size_t o = cnt[(ka[i] >> sh) & 255u]++;
                kb[o] = ka[i];
                vb[o] = va[i];
            }
            ka.swap(kb);
            va.swap(vb);
        }
        std::memcpy(keys_out, ka.data(), sizeof(K) * n);
        std::memcpy(vals_out, va.data(), sizeof(V) * n);
        return 0;
    }
};
}  // namespace cub
