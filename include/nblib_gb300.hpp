/*
 * nblib_gb300.hpp -- nblib's ForceCalculator on the GB300 engine (C++17, header only).
 *
 * Mirrors the public surface of nblib that drives the nonbonded path:
 *   ForceCalculator(const SimulationState&, const NBKernelOptions&)   api/nblib/forcecalculator.h:78
 *   void compute(ArrayRef<const Vec3> coordinates, ArrayRef<Vec3> forces)   forcecalculator.h:90
 *   void updatePairList(ArrayRef<const int>, ArrayRef<Vec3>, const Box&)   forcecalculator.h:101
 *   NBKernelOptions, CoulombType, CombinationRule, SimdKernels       api/nblib/kerneloptions.h:56-113
 *   InputException                                                  api/nblib/exception.h
 * with the same argument meaning and error behaviour: forces are overwritten
 * (gmxcalculator.cpp:76-82), triclinic boxes and bad input raise InputException.
 * Everything runs through the C ABI of include/nbnxm_gb300.h (link
 * libnbnxm_gb300.so); nothing here touches CUDA directly.
 *
 * The topology is reduced to what the nonbonded path reads from nblib's
 * Topology (topology.h:72-98): per-particle type ids and charges, per-type
 * C6/C12 (or an explicit type-pair table) and the exclusion lists.
 */
#ifndef NBLIB_GB300_HPP
#define NBLIB_GB300_HPP

#include <array>
#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "nbnxm_gb300.h"

namespace nblib_gb300
{

using real = float;
//! gmx::RVec layout: three floats per particle
using Vec3 = std::array<real, 3>;

//! Non-owning view, the role gmx::ArrayRef plays in nblib's signatures
template<typename T>
class ArrayRef
{
public:
    ArrayRef() = default;
    ArrayRef(T* data, std::size_t size) : data_(data), size_(size) {}
    template<typename V>
    ArrayRef(V& v) : data_(v.data()), size_(v.size())  // NOLINT(google-explicit-constructor)
    {
    }
    T*          data() const { return data_; }
    std::size_t size() const { return size_; }
    T&          operator[](std::size_t i) const { return data_[i]; }
    T*          begin() const { return data_; }
    T*          end() const { return data_ + size_; }

private:
    T*          data_ = nullptr;
    std::size_t size_ = 0;
};

//! nblib::InputException (api/nblib/exception.h)
class InputException : public std::runtime_error
{
public:
    explicit InputException(const std::string& what) : std::runtime_error(what) {}
};

//! A failure of the device engine (out of memory, CUDA error, bounded wait gave up)
class GpuException : public std::runtime_error
{
public:
    GpuException(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

enum class SimdKernels : int
{
    SimdAuto,
    SimdNo,
    Simd4XM,
    Simd2XMM,
    Count
};

enum class CombinationRule : int
{
    Geometric,
    LorentzBerthelot,
    None,
    Count
};

enum class CoulombType : int
{
    Pme,
    Cutoff,
    ReactionField,
    Count
};

//! nblib::NBKernelOptions with the GPU list parameters appended
struct NBKernelOptions
{
    bool            useGpu                 = true;  // the engine is the GPU path
    int             numOpenMPThreads       = 1;     // accepted, unused
    SimdKernels     nbnxmSimd              = SimdKernels::SimdAuto;  // accepted, unused
    CombinationRule ljCombinationRule      = CombinationRule::Geometric;
    bool            useHalfLJOptimization  = false;  // accepted, unused
    real            pairlistCutoff         = 1.0f;
    bool            computeVirialAndEnergy = false;
    CoulombType     coulombType            = CoulombType::Pme;
    bool            useTabulatedEwaldCorr  = false;  // the GPU kernel evaluates erfc analytically
    int             numIterations          = 100;
    bool            cyclesPerPair          = false;
    real            timestep               = 0.001f;
    // GPU list parameters (PairlistParams, pairlistparams.h:115-141)
    real   rcoulomb      = 0.0f;  // <= 0: pairlistCutoff (nblib's rc = rvdw = rlist)
    real   rlistInner    = 0.0f;  // <= 0: no dynamic pruning radius
    int    nstlist       = 10;
    int    nstlistPrune  = 0;
    real   ewaldRtol     = 1e-5f;
    real   epsilonRf     = 1.0f;
    bool   useEwaldShift = false;
    int    device        = 0;
};

//! Rectangular box (nblib::Box with a diagonal matrix)
class Box
{
public:
    explicit Box(real l) : Box(l, l, l) {}
    Box(real x, real y, real z) : edges_{ x, y, z }
    {
        for (real e : edges_)
        {
            if (!(e > 0.0f) || !std::isfinite(e))
            {
                throw InputException("box edges must be positive and finite");
            }
        }
    }
    real x() const { return edges_[0]; }
    real y() const { return edges_[1]; }
    real z() const { return edges_[2]; }
    bool operator==(const Box& o) const { return edges_ == o.edges_; }
    bool operator!=(const Box& o) const { return !(*this == o); }

private:
    std::array<real, 3> edges_;
};

//! What the nonbonded path reads from nblib::Topology
class Topology
{
public:
    //! Per-type C6/C12 combined by rule (interactions.cpp:83-93 for Geometric;
    //! Lorentz-Berthelot from sigma = (C12/C6)^(1/6), epsilon = C6^2/(4 C12)).
    Topology(std::vector<int> typeIds, std::vector<real> charges, const std::vector<real>& c6PerType,
             const std::vector<real>& c12PerType, CombinationRule rule,
             std::vector<std::vector<int>> exclusions = {}) :
        types_(std::move(typeIds)), charges_(std::move(charges))
    {
        const std::size_t nt = c6PerType.size();
        if (c12PerType.size() != nt)
        {
            throw InputException("C6 and C12 need one entry per particle type");
        }
        nbfp_.resize(2 * nt * nt);
        for (std::size_t a = 0; a < nt; a++)
        {
            for (std::size_t b = 0; b < nt; b++)
            {
                if (rule == CombinationRule::Geometric)
                {
                    // single precision like nblib's combineNonbondedParameters and c6factor/c12factor
                    nbfp_[2 * (a * nt + b)]     = std::sqrt(c6PerType[a] * c6PerType[b]) * real(6);
                    nbfp_[2 * (a * nt + b) + 1] = std::sqrt(c12PerType[a] * c12PerType[b]) * real(12);
                    continue;
                }
                if (rule != CombinationRule::LorentzBerthelot)
                {
                    throw InputException("unknown LJ Combination rule specified");
                }
                auto se = [](double c6i, double c12i) {
                    if (c6i <= 0.0 || c12i <= 0.0)
                    {
                        return std::pair<double, double>(0.0, 0.0);
                    }
                    return std::pair<double, double>(std::pow(c12i / c6i, 1.0 / 6.0), c6i * c6i / (4.0 * c12i));
                };
                const auto   pa  = se(c6PerType[a], c12PerType[a]);
                const auto   pb  = se(c6PerType[b], c12PerType[b]);
                const double sig = 0.5 * (pa.first + pb.first);
                const double eps = std::sqrt(pa.second * pb.second);
                const double s6  = std::pow(sig, 6.0);
                const double c6  = 4.0 * eps * s6;
                const double c12 = c6 * s6;
                nbfp_[2 * (a * nt + b)]     = (real)(6.0 * c6);
                nbfp_[2 * (a * nt + b) + 1] = (real)(12.0 * c12);
            }
        }
        numTypes_ = (int)nt;
        setExclusions(exclusions);
        validate();
    }

    //! Explicit type-pair table {6*C6, 12*C12} (nblib's nonbondedParameters_, gmxsetup.cpp:143-166)
    Topology(std::vector<int> typeIds, std::vector<real> charges, int numTypes, std::vector<real> nbfp,
             std::vector<std::vector<int>> exclusions = {}) :
        types_(std::move(typeIds)), charges_(std::move(charges)), nbfp_(std::move(nbfp)), numTypes_(numTypes)
    {
        setExclusions(exclusions);
        validate();
    }

    int                      numParticles() const { return (int)types_.size(); }
    const std::vector<int>&  getParticleTypeIdOfAllParticles() const { return types_; }
    const std::vector<real>& getCharges() const { return charges_; }
    int                      numParticleTypes() const { return numTypes_; }
    const std::vector<real>& nonbondedParameters() const { return nbfp_; }
    const std::vector<int>&  exclusionIndex() const { return exclIndex_; }
    const std::vector<int>&  exclusionList() const { return exclList_; }

private:
    void setExclusions(const std::vector<std::vector<int>>& exclusions)
    {
        const std::size_t n = types_.size();
        exclIndex_.assign(n + 1, 0);
        for (std::size_t i = 0; i < n; i++)
        {
            const std::size_t m = i < exclusions.size() ? exclusions[i].size() : 0;
            exclIndex_[i + 1]   = exclIndex_[i] + (int)m;
            for (std::size_t k = 0; k < m; k++)
            {
                exclList_.push_back(exclusions[i][k]);
            }
        }
        if (exclList_.empty())
        {
            exclList_.push_back(0);  // a valid pointer for an empty list
        }
    }
    void validate() const
    {
        if (charges_.size() != types_.size())
        {
            throw InputException("one charge per particle is required");
        }
        if (nbfp_.size() != 2 * (std::size_t)numTypes_ * numTypes_)
        {
            throw InputException("the type-pair table needs 2 * numTypes^2 entries");
        }
    }

    std::vector<int>  types_;
    std::vector<real> charges_;
    std::vector<real> nbfp_;
    int               numTypes_ = 0;
    std::vector<int>  exclIndex_;
    std::vector<int>  exclList_;
};

//! nblib::SimulationState (simulationstate.h:63-100)
class SimulationState
{
public:
    SimulationState(const std::vector<Vec3>& coordinates, const std::vector<Vec3>& velocities,
                    const std::vector<Vec3>& forces, Box box, Topology topology) :
        coordinates_(coordinates), velocities_(velocities), forces_(forces), box_(box), topology_(std::move(topology))
    {
        if ((int)coordinates_.size() != topology_.numParticles())
        {
            throw InputException("coordinates and topology disagree on the number of particles");
        }
        for (const Vec3& x : coordinates_)
        {
            for (real c : x)
            {
                if (!std::isfinite(c))
                {
                    throw InputException("non-finite coordinate");
                }
            }
        }
    }
    const Topology&          topology() const { return topology_; }
    Box                      box() const { return box_; }
    std::vector<Vec3>&       coordinates() { return coordinates_; }
    const std::vector<Vec3>& coordinates() const { return coordinates_; }
    std::vector<Vec3>&       velocities() { return velocities_; }
    std::vector<Vec3>&       forces() { return forces_; }

private:
    std::vector<Vec3> coordinates_;
    std::vector<Vec3> velocities_;
    std::vector<Vec3> forces_;
    Box               box_;
    Topology          topology_;
};

//! nblib::ForceCalculator on one GPU (forcecalculator.h:75-109)
class ForceCalculator
{
public:
    ForceCalculator(const SimulationState& system, const NBKernelOptions& options) :
        topology_(system.topology()), options_(options), box_(system.box())
    {
        if (options.coulombType == CoulombType::Count)
        {
            throw InputException("invalid Coulomb type");
        }
        create(system.coordinates().data(), box_);
    }
    ~ForceCalculator() { nbx_destroy(handle_); }
    ForceCalculator(const ForceCalculator&) = delete;
    ForceCalculator& operator=(const ForceCalculator&) = delete;

    //! Zeroes and fills forces; energies and virial when options request them
    void compute(ArrayRef<const Vec3> coordinates, ArrayRef<Vec3> forces)
    {
        const std::size_t n = (std::size_t)topology_.numParticles();
        if (coordinates.size() != n || forces.size() != n)
        {
            throw InputException("coordinates and forces must hold one Vec3 per particle");
        }
        double* e = options_.computeVirialAndEnergy ? energies_.data() : nullptr;
        double* v = options_.computeVirialAndEnergy ? virial_.data() : nullptr;
        check(nbx_compute(handle_, coordinates.data()->data(), forces.data()->data(), e, v));
    }

    //! Re-grids and rebuilds the pair list (the particle info flags are accepted for
    //! signature parity: every particle has LJ and charge, gmxsetup.cpp:132-141)
    void updatePairList(ArrayRef<const int> particleInfoAllVdW, ArrayRef<Vec3> coordinates, const Box& box)
    {
        (void)particleInfoAllVdW;
        if (coordinates.size() != (std::size_t)topology_.numParticles())
        {
            throw InputException("coordinates must hold one Vec3 per particle");
        }
        if (box != box_)
        {
            // the grid and shift vectors follow the box: start over with the new one
            nbx_destroy(handle_);
            handle_ = nullptr;
            box_    = box;
            create(coordinates.data(), box_);
            return;
        }
        check(nbx_update_pairlist(handle_, coordinates.data()->data()));
    }

    //! {LJ, Coulomb} energies (kJ/mol) of the last compute with computeVirialAndEnergy
    const std::array<double, 2>& energies() const { return energies_; }
    //! Virial (row-major 3x3, kJ/mol) of the last compute with computeVirialAndEnergy
    const std::array<double, 9>& virial() const { return virial_; }
    //! The underlying C-ABI handle (device-pointer entry points)
    nbx_handle* handle() const { return handle_; }

private:
    void create(const Vec3* coordinates, const Box& box)
    {
        nbx_system_desc d{};
        d.num_atoms  = topology_.numParticles();
        d.x          = coordinates->data();
        d.q          = topology_.getCharges().data();
        d.type       = topology_.getParticleTypeIdOfAllParticles().data();
        d.num_types  = topology_.numParticleTypes();
        d.nbfp       = topology_.nonbondedParameters().data();
        d.excl_index = topology_.exclusionIndex().data();
        d.excl_list  = topology_.exclusionList().data();
        d.box[0]     = box.x();
        d.box[1]     = box.y();
        d.box[2]     = box.z();
        nbx_options o;
        nbx_default_options(&o);
        o.coulomb         = (int)options_.coulombType;  // same numbering as nblib
        o.rlist           = options_.pairlistCutoff;
        o.rcoulomb        = options_.rcoulomb > 0.0f ? options_.rcoulomb : options_.pairlistCutoff;
        o.rlist_inner     = options_.rlistInner;
        o.ewald_rtol      = options_.ewaldRtol;
        o.epsilon_rf      = options_.epsilonRf;
        o.use_ewald_shift = options_.useEwaldShift ? 1 : 0;
        o.nstlist         = options_.nstlist;
        o.nstlist_prune   = options_.nstlistPrune;
        o.compute_energy  = options_.computeVirialAndEnergy ? 1 : 0;
        const int rc      = nbx_create(&d, &o, options_.device, &handle_);
        if (rc != NBX_OK)
        {
            const std::string msg = nbx_last_error(nullptr);
            if (rc == NBX_ERR_INVALID_INPUT)
            {
                throw InputException(msg);
            }
            throw GpuException(rc, msg);
        }
    }
    void check(int rc) const
    {
        if (rc == NBX_OK)
        {
            return;
        }
        const std::string msg = nbx_last_error(handle_);
        if (rc == NBX_ERR_INVALID_INPUT)
        {
            throw InputException(msg);
        }
        throw GpuException(rc, msg);
    }

    Topology               topology_;
    NBKernelOptions        options_;
    Box                    box_;
    nbx_handle*            handle_ = nullptr;
    std::array<double, 2>  energies_{};
    std::array<double, 9>  virial_{};
};

} // namespace nblib_gb300

#endif // NBLIB_GB300_HPP
