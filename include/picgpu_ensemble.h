/*
 * picgpu_ensemble.h -- batched ensembles of independent cases in one
 * context, stepped by a CUDA graph (no picFoam counterpart: picFoam runs
 * one case per process).
 *
 * picgpu_ensemble_create replicates one block mesh n_cases times as
 * disjoint copies (cells, points and boundary faces of case k follow those of
 * case k - 1), so every kernel of a step processes all cases in one launch;
 * tet index 12 * (k * cells_per_case + c) + local tet addresses cell c of case
 * k.  picgpu_step_graph runs steps as a captured CUDA graph of
 * steps_per_graph steps in which particle counts, MCC candidates and
 * secondaries stay on the device (no host synchronisation inside a replay).
 * It needs the FP32 form (PICGPU_PREC_MIXED) and MaxwellSolver none.
 */
#ifndef PICGPU_ENSEMBLE_H
#define PICGPU_ENSEMBLE_H

#include "picgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

picgpu_status picgpu_ensemble_create(const picgpu_mesh_desc* one_case, int n_cases, const picgpu_config* cfg,
                                     picgpu_ctx** out);
/* Applied field of every case, E[n_cases][3] [V/m] (MaxwellSolver none). */
picgpu_status picgpu_ensemble_set_efield(picgpu_ctx* ctx, const double* E);
/* Per case, over the particles of one species: out[k][0] count, [1..3]
 * sum of velocity components, [4] sum of |U|^2; ionisations[k]: MCC
 * ionisation events since creation (may be NULL). */
picgpu_status picgpu_ensemble_case_stats(picgpu_ctx* ctx, int species, double* out, int64_t* ionisations);

/* nsteps steps (a multiple of steps_per_graph) through CUDA graphs of
 * steps_per_graph steps.  The first call tunes the launch shapes (see
 * picgpu_graph_tuning) on its first replays. */
picgpu_status picgpu_step_graph(picgpu_ctx* ctx, int nsteps, int steps_per_graph, picgpu_step_stats* stats);
/* The launch shapes chosen by the tuner: move blocks per SM, MCC threads
 * per block, and the measured ns per particle-step of each candidate tried
 * (times[n_times], move candidates first). */
picgpu_status picgpu_graph_tuning(picgpu_ctx* ctx, int* move_blocks_per_sm, int* mcc_block, double* times,
                                  int n_times);

#ifdef __cplusplus
}
#endif
#endif
