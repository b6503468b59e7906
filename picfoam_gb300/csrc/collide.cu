// collide.cu -- collision step: cell sort, null-collision MCC, Coulomb.
#include "collide.h"

namespace pgd {

__constant__ TetConst c_tetC;

cudaError_t collide_set_tables(const TetConst& t) { return cudaMemcpyToSymbol(c_tetC, &t, sizeof t); }

int collide_init(CollideState& st, const picgpu_config& cfg, const DMesh& m, cudaStream_t s, std::string* msg) {
    (void)m;
    (void)s;
    st.enabled = cfg.mcc.enabled || cfg.coulomb.enabled;
    if (st.enabled) {
        *msg = "collisions are not available in this build";
        return PICGPU_NOT_SUPPORTED;
    }
    return PICGPU_OK;
}

void collide_free(CollideState& st) { (void)st; }

int run_collisions(CollideState& st, const CollideArgs& a, int64_t counts[8], long newn[], int swapped[],
                   std::string* msg, int64_t* launches, double* phase_ms) {
    (void)st; (void)counts; (void)swapped; (void)launches; (void)phase_ms;
    for (int s = 0; s < a.n_species; ++s) newn[s] = a.n[s];
    *msg = "collisions are not available in this build";
    return PICGPU_NOT_SUPPORTED;
}

}  // namespace pgd
