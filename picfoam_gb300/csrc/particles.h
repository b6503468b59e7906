// particles.h -- particle store maintenance (host declarations).
#pragma once

#include "common.cuh"

namespace pgd {

long compact_blocks(long n);
// Stable compaction of src (n slots, removed ones have tet < 0) into dst.
// scan needs compact_blocks(n) + 1 ints.  Synchronises the stream.
cudaError_t compact_species(const DSpecies& src, const DSpecies& dst, long n, bool mixed, int* scan,
                            long* kept, cudaStream_t s);

// Host-facing row-major copies of a store: tet range check, rows (n x 3
// FP64) -> columns (FP32 or FP64), columns -> rows.
void launch_check_tets(const int32_t* tet, long n, long long ntet, int* bad, cudaStream_t s);
void launch_scatter_rows(const int32_t* tet, const double* bary, const double* U, long n, const DSpecies& dst,
                         bool fp32, cudaStream_t s);
// Parcels [from, to) of a store with per-parcel attributes get the
// defaults of a new parcel (PICCloud::addNewParcel): the species weight and
// charge modifier 1.  No-op for a store without attributes.
void launch_fill_attributes(const DSpecies& d, long from, long to, double weight, cudaStream_t s);
void launch_gather_rows(const DSpecies& src, long n, bool fp32, int32_t* tet, double* bary, double* U,
                        cudaStream_t s);

}  // namespace pgd
