// Stand-in for the third-party `simultaneous-sort` header (vcpkg port `simultaneous-sort`, pinned only
// through the reference's vcpkg baseline; its source is not part of the reference tree), oracle
// build only. Published behaviour: sort_with(comp, keys, values...) sorts `keys` by `comp` and applies
// the same permutation to every `values` vector. ParticlesToDensity uses it only in vector mode to
// order the compacted output grid (ParticlesToDensity.cpp:689); it affects output order, not values.
// This stand-in uses a stable sort; the ordering of equal keys is therefore this file's choice.
#pragma once

#include <algorithm>
#include <cstddef>
#include <numeric>
#include <vector>

template<class Comp, class K, class... V>
void sort_with(Comp comp, std::vector<K>& keys, std::vector<V>&... values) {
    std::vector<std::size_t> perm(keys.size());
    std::iota(perm.begin(), perm.end(), std::size_t{0});
    std::stable_sort(perm.begin(), perm.end(), [&](std::size_t a, std::size_t b) { return comp(keys[a], keys[b]); });
    auto apply = [&perm](auto& v) {
        auto copy = v;
        for (std::size_t i = 0; i < perm.size() && i < v.size(); ++i)
            v[i] = copy[perm[i]];
    };
    apply(keys);
    (apply(values), ...);
}
