// particles.h -- particle store maintenance (host declarations).
#pragma once

#include "common.cuh"

namespace pgd {

long compact_blocks(long n);
// Stable compaction of src (n slots, removed ones have tet < 0) into dst.
// scan needs compact_blocks(n) + 1 ints.  Synchronises the stream.
cudaError_t compact_species(const DSpecies& src, const DSpecies& dst, long n, bool mixed, int* scan,
                            long* kept, cudaStream_t s);

}  // namespace pgd
