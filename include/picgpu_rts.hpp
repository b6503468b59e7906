/* picgpu_rts.hpp -- picFoam's run-time selection over the picgpu C ABI (C++17,
 * header only, no OpenFOAM types).
 *
 * picFoam selects each sub-model of PICCloud by the TypeName a dictionary
 * keyword names (picProperties: `ParticlePusher Boris;`, `FieldWeigthing
 * VolumeWeighting;` ...), through OpenFOAM's run-time selection tables
 * (declareRunTimeSelectionTable / addToRunTimeSelectionTable, e.g.
 * PICMCCFVM/parcels/derived/picParcel/makeParticlePusher.C:40-47 and the
 * TypeName of each model, BorisPusher.H:62).  Here each selectable model of
 * the GPU path is a class with picFoam's TypeName, registered in a table of
 * its model family under that name, whose apply() writes the model's choice
 * into a picgpu_config.  A picFoam build that keeps its dictionaries calls
 *
 *     picgpu::rts::select(cfg, "ParticlePusher", dict.lookup("ParticlePusher"));
 *
 * for each keyword, then creates the context with picgpu_create and steps
 * it with picgpu::rts::Cloud::evolve (PICCloud::evolve, PICCloud.C:1426-1471).
 * An unknown TypeName throws std::invalid_argument listing the valid ones,
 * as OpenFOAM's FatalError lists the table.
 */
#ifndef PICGPU_RTS_HPP
#define PICGPU_RTS_HPP

#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "picgpu.h"

namespace picgpu {
namespace rts {

// A model family (ParticlePusher, FieldWeigthing, ...): TypeName -> model.
class Model {
public:
    virtual ~Model() = default;
    virtual const char* type() const = 0;
    virtual void apply(picgpu_config& cfg) const = 0;
};

using Factory = std::function<std::unique_ptr<Model>()>;

// The table of one family, filled by the Register objects below (static
// initialisation, as addToRunTimeSelectionTable does).
inline std::map<std::string, std::map<std::string, Factory>>& tables() {
    static std::map<std::string, std::map<std::string, Factory>> t;
    return t;
}

template <class M>
struct Register {
    explicit Register(const char* family) { tables()[family][M::typeName] = [] { return std::make_unique<M>(); }; }
};

// Model::New: the model of `family` called `typeName`.
inline std::unique_ptr<Model> New(const std::string& family, const std::string& typeName) {
    auto f = tables().find(family);
    if (f == tables().end()) throw std::invalid_argument("unknown model family " + family);
    auto m = f->second.find(typeName);
    if (m == f->second.end()) {
        std::string valid;
        for (const auto& kv : f->second) valid += " " + kv.first;
        throw std::invalid_argument("Unknown " + family + " type " + typeName + "; valid types:" + valid);
    }
    return m->second();
}

// Select the model `typeName` of `family` into cfg; returns its TypeName.
inline std::string select(picgpu_config& cfg, const std::string& family, const std::string& typeName) {
    const std::unique_ptr<Model> m = New(family, typeName);
    m->apply(cfg);
    return m->type();
}

// The TypeNames a family offers.
inline std::vector<std::string> types(const std::string& family) {
    std::vector<std::string> out;
    for (const auto& kv : tables()[family]) out.push_back(kv.first);
    return out;
}

#define PICGPU_RTS_MODEL(Class, Family, Name, Body)                               \
    struct Class : Model {                                                          \
        static constexpr const char* typeName = Name;                               \
        const char* type() const override { return typeName; }                      \
        void apply(picgpu_config& cfg) const override { Body; }                     \
    };                                                                              \
    inline const Register<Class> register_##Class{Family};

// ParticlePusher (SM/ParticlePusher/*): NoPush "none", BorisPusher "Boris",
// BorisNRPusher "BorisNR", VayPusher "Vay", HigueraCary "HigueraCary"
PICGPU_RTS_MODEL(NoPush, "ParticlePusher", "none", cfg.pusher = PICGPU_PUSHER_NONE)
PICGPU_RTS_MODEL(BorisPusher, "ParticlePusher", "Boris", cfg.pusher = PICGPU_PUSHER_BORIS)
PICGPU_RTS_MODEL(BorisNRPusher, "ParticlePusher", "BorisNR", cfg.pusher = PICGPU_PUSHER_BORIS_NR)
PICGPU_RTS_MODEL(VayPusher, "ParticlePusher", "Vay", cfg.pusher = PICGPU_PUSHER_VAY)
PICGPU_RTS_MODEL(HigueraCaryPusher, "ParticlePusher", "HigueraCary", cfg.pusher = PICGPU_PUSHER_HIGUERA_CARY)

// FieldWeigthing (SM/FieldWeigthing/*) and ChargeDistribution
// (SM/ChargeDistribution/*): "CellAverage", "VolumeWeighting"
PICGPU_RTS_MODEL(CellAverageFW, "FieldWeigthing", "CellAverage", cfg.field_weighting = PICGPU_WEIGHTING_CELL_AVERAGE)
PICGPU_RTS_MODEL(VolumeWeightingFW, "FieldWeigthing", "VolumeWeighting",
                 cfg.field_weighting = PICGPU_WEIGHTING_VOLUME)
PICGPU_RTS_MODEL(CellAverage, "ChargeDistribution", "CellAverage",
                 cfg.charge_distribution = PICGPU_WEIGHTING_CELL_AVERAGE)
PICGPU_RTS_MODEL(VolumeWeighting, "ChargeDistribution", "VolumeWeighting",
                 cfg.charge_distribution = PICGPU_WEIGHTING_VOLUME)

// MaxwellSolver (SM/MaxwellSolver/*): "none", ElectroStaticSolver "ElectroStatic"
PICGPU_RTS_MODEL(NoMaxwellSolver, "MaxwellSolver", "none", cfg.maxwell_solver = PICGPU_MAXWELL_NONE)
PICGPU_RTS_MODEL(ElectroStaticSolver, "MaxwellSolver", "ElectroStatic",
                 cfg.maxwell_solver = PICGPU_MAXWELL_ELECTROSTATIC)

// CoulombCollisionModel (NoCoulombCollision "none", NanbuCollision "Nanbu",
// PerezRelativisticCollision "Perez"), its PairingAlgorithm
// (NanbuYonemura, TakizukaAbe), WeightCorrectionModel (none, Nanbu,
// SentokuKempNR, SentokuKemp) and IonizationModel (none, Perez: the
// coefficients go to cfg.perez.ion[])
PICGPU_RTS_MODEL(NoCoulombCollision, "CoulombCollisionModel", "none", cfg.coulomb.enabled = 0)
PICGPU_RTS_MODEL(NanbuCollision, "CoulombCollisionModel", "Nanbu",
                 (cfg.coulomb.enabled = 1, cfg.coulomb.collide = PICGPU_COLLIDE_NANBU))
PICGPU_RTS_MODEL(PerezRelativisticCollision, "CoulombCollisionModel", "Perez",
                 (cfg.coulomb.enabled = 1, cfg.coulomb.collide = PICGPU_COLLIDE_PEREZ))
PICGPU_RTS_MODEL(NanbuYonemuraPairing, "PairingAlgorithm", "NanbuYonemura",
                 cfg.coulomb.pairing = PICGPU_PAIRING_NANBU_YONEMURA)
PICGPU_RTS_MODEL(TakizukaAbePairing, "PairingAlgorithm", "TakizukaAbe",
                 cfg.coulomb.pairing = PICGPU_PAIRING_TAKIZUKA_ABE)
PICGPU_RTS_MODEL(NoCorrection, "WeightCorrectionModel", "none",
                 cfg.coulomb.weight_correction = PICGPU_WEIGHT_CORRECTION_NONE)
PICGPU_RTS_MODEL(NanbuCorrection, "WeightCorrectionModel", "Nanbu",
                 cfg.coulomb.weight_correction = PICGPU_WEIGHT_CORRECTION_NANBU)
PICGPU_RTS_MODEL(SentokuKempNRCorrection, "WeightCorrectionModel", "SentokuKempNR",
                 cfg.coulomb.weight_correction = PICGPU_WEIGHT_CORRECTION_SENTOKU_KEMP_NR)
PICGPU_RTS_MODEL(SentokuKempCorrection, "WeightCorrectionModel", "SentokuKemp",
                 cfg.coulomb.weight_correction = PICGPU_WEIGHT_CORRECTION_SENTOKU_KEMP)
PICGPU_RTS_MODEL(NoIonization, "IonizationModel", "none", cfg.perez.enabled = 0)
PICGPU_RTS_MODEL(PerezIonizationModel, "IonizationModel", "Perez", cfg.perez.enabled = 1)

// ParticleMerging (NoMerging "none", PairMerging; the coefficients go to
// cfg.merging)
PICGPU_RTS_MODEL(NoMerging, "ParticleMerging", "none", cfg.merging.enabled = 0)
PICGPU_RTS_MODEL(PairMerging, "ParticleMerging", "PairMerging", cfg.merging.enabled = 1)

// BinaryCollisionModel (NoBinaryCollision "none", IsotropicScattering; the
// coefficients go to cfg.binary)
PICGPU_RTS_MODEL(NoBinaryCollision, "BinaryCollisionModel", "none", cfg.binary.enabled = 0)
PICGPU_RTS_MODEL(IsotropicScattering, "BinaryCollisionModel", "IsotropicScattering", cfg.binary.enabled = 1)

#undef PICGPU_RTS_MODEL

// The PICCloud of one context: evolve() is PICCloud::evolve (injection,
// move, collisions, charge, field solve, circuit and merging in picFoam's
// order), info() its step statistics; the context is released with the
// object.
class Cloud {
public:
    Cloud(const picgpu_mesh_desc& mesh, const picgpu_config& cfg) {
        const picgpu_status s = picgpu_create(&mesh, &cfg, &ctx_);
        if (s != PICGPU_OK) {
            const std::string why = ctx_ ? picgpu_last_error(ctx_) : "";
            if (ctx_) picgpu_destroy(ctx_);
            ctx_ = nullptr;
            throw std::runtime_error("picgpu_create failed (" + std::to_string(int(s)) + "): " + why);
        }
    }
    ~Cloud() {
        if (ctx_) picgpu_destroy(ctx_);
    }
    Cloud(const Cloud&) = delete;
    Cloud& operator=(const Cloud&) = delete;

    picgpu_ctx* context() const { return ctx_; }

    void setParticles(int species, size_t n, const int32_t* tet, const double* bary, const double* U) {
        check(picgpu_set_particles(ctx_, species, n, tet, bary, U), "picgpu_set_particles");
    }
    void initialiseFields() { check(picgpu_initialise_fields(ctx_), "picgpu_initialise_fields"); }
    const picgpu_step_stats& evolve(int steps = 1) {
        check(picgpu_step(ctx_, steps, &stats_), "picgpu_step");
        return stats_;
    }
    const picgpu_step_stats& info() const { return stats_; }

private:
    void check(picgpu_status s, const char* what) const {
        if (s != PICGPU_OK)
            throw std::runtime_error(std::string(what) + " failed (" + std::to_string(int(s)) +
                                     "): " + picgpu_last_error(ctx_));
    }
    picgpu_ctx* ctx_ = nullptr;
    picgpu_step_stats stats_{};
};

}  // namespace rts
}  // namespace picgpu

#endif /* PICGPU_RTS_HPP */
