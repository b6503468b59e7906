// rts_driver.cpp -- a compiled C++ host of the picgpu library: picFoam's
// PICCloud time loop (solver/picFoam/picFoam.C: evolve every step) with
// the sub-models chosen by their picFoam TypeNames through the run-time
// selection tables of picgpu_rts.hpp.
//
//   picgpu_rts_driver IN OUT STEPS Family=TypeName ...
//
// IN holds the case: the picgpu_mesh_desc and picgpu_config structs as
// bytes (a config without cross-section tables), then per species the
// parcel count (int64) and its tet (int32), barycentric (3 double) and
// velocity (3 double) arrays.  Every Family=TypeName argument is selected
// into the config (ParticlePusher=Vay, FieldWeigthing=CellAverage, ...)
// before picgpu_create.  After initialising the fields and STEPS calls of
// evolve(), OUT receives the last step's picgpu_step_stats as bytes and
// then, per species, the parcels in the same layout.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

#include "picgpu_rts.hpp"

namespace {

template <class T>
bool get(std::ifstream& f, T* p, size_t n = 1) {
    return bool(f.read(reinterpret_cast<char*>(p), std::streamsize(n * sizeof(T))));
}

template <class T>
void put(std::ofstream& f, const T* p, size_t n = 1) {
    f.write(reinterpret_cast<const char*>(p), std::streamsize(n * sizeof(T)));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::cerr << "usage: " << argv[0] << " IN OUT STEPS [Family=TypeName ...]\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    picgpu_mesh_desc mesh;
    picgpu_config cfg;
    if (!get(in, &mesh) || !get(in, &cfg)) {
        std::cerr << "cannot read the case from " << argv[1] << "\n";
        return 2;
    }
    // the tables of the input config are not in this process
    cfg.mcc.xs_energy = cfg.mcc.xs_elastic = cfg.mcc.xs_excitation = cfg.mcc.xs_ionization = nullptr;
    cfg.ion_mcc.xs_energy = cfg.ion_mcc.xs_elastic = cfg.ion_mcc.xs_charge_exchange = nullptr;
    const int steps = std::atoi(argv[3]);
    try {
        for (int k = 4; k < argc; ++k) {
            const std::string a = argv[k];
            const size_t eq = a.find('=');
            if (eq == std::string::npos) throw std::invalid_argument("expected Family=TypeName, got " + a);
            const std::string chosen = picgpu::rts::select(cfg, a.substr(0, eq), a.substr(eq + 1));
            std::cout << a.substr(0, eq) << " " << chosen << "\n";
        }
        picgpu::rts::Cloud cloud(mesh, cfg);
        for (int s = 0; s < cfg.n_species; ++s) {
            int64_t n = 0;
            if (!get(in, &n)) throw std::runtime_error("cannot read the parcels");
            std::vector<int32_t> tet(static_cast<size_t>(n));
            std::vector<double> bary(3 * static_cast<size_t>(n)), U(3 * static_cast<size_t>(n));
            if (!get(in, tet.data(), tet.size()) || !get(in, bary.data(), bary.size()) || !get(in, U.data(), U.size()))
                throw std::runtime_error("cannot read the parcels");
            cloud.setParticles(s, size_t(n), tet.data(), bary.data(), U.data());
        }
        cloud.initialiseFields();
        picgpu_step_stats st{};
        for (int k = 0; k < steps; ++k) st = cloud.evolve(1);
        std::ofstream out(argv[2], std::ios::binary);
        put(out, &st);
        for (int s = 0; s < cfg.n_species; ++s) {
            size_t n = 0;
            if (picgpu_count_particles(cloud.context(), s, &n) != PICGPU_OK) throw std::runtime_error("count");
            std::vector<int32_t> tet(n);
            std::vector<double> bary(3 * n), U(3 * n);
            size_t got = 0;
            if (picgpu_get_particles(cloud.context(), s, n, tet.data(), bary.data(), U.data(), &got) != PICGPU_OK)
                throw std::runtime_error("get_particles");
            const int64_t m = int64_t(got);
            put(out, &m);
            put(out, tet.data(), got);
            put(out, bary.data(), 3 * got);
            put(out, U.data(), 3 * got);
        }
        std::cout << "steps " << steps << " pcg_iterations " << st.pcg_iterations << "\n";
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    return 0;
}
