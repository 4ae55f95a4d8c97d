/*
 * alias_ref.cpp — C entry point around the reference's own alias-table builder
 * (src/util/AliasTable.h, DiscreteSampler1D<float>::build), compiled from the reference
 * source in place (-I REFERENCE/src) by oracle/ref/make_ref.py.
 *
 * TEST INFRASTRUCTURE (oracle): pins grisBuildLightTable and the oracle's table semantics.
 */
#include <stdint.h>
#include <vector>
#include "util/AliasTable.h"

extern "C" void aliasref_build(const float* distribution, uint32_t n, float* prob, uint32_t* failId) {
    std::vector<float> d(distribution, distribution + n);
    DiscreteSampler1D<float> s(d);
    for (uint32_t i = 0; i <= n; i++) { prob[i] = s.binomDistribs[i].prob; failId[i] = s.binomDistribs[i].failId; }
}
