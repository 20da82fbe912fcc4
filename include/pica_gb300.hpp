// pica_gb300.hpp -- header-only C++ mirror of pica's hot-path classes over the
// pica_gb300 C ABI (pica_gb300.h).
//
// pica's host loop constructs a YeeGrid, an EnsembleSupercells of
// ParticleArraySoA<Particle3d>, a BorisPusher, and per supercell a
// FieldInterpolatorCICSupercell and a CurrentDepositorCICSupercell, then calls
// get / push / deposit per particle and YeeSolver::updateB/updateE per step.
// Here the same names stand for device-resident objects and each operator
// acts on every particle at once:
//
//   pica:                                            pica_gb300:
//   YeeGrid<Three,double> grid(origin, step, size)   Simulation sim(config); auto& grid = sim.grid();
//   grid.ex(i,j,k) = v                               grid.ex(i,j,k) = v; ...; grid.upload();
//   EnsembleSupercells<PA> ens(min, max, N, S)        auto& ens = sim.ensemble();
//   ens.add(particle)                                 ens.add(particle); ...; ens.upload();
//   BorisPusher<Particle3d,double> pusher(dt)         (dt and ParticleTypes are in the config)
//   for each supercell, particle: fi.get; pusher.push;  pushSupercells(sim);      // one call
//     cd.deposit; ~cd                                 ens.migrate();
//   YeeSolver().updateB(grid, dt)                      YeeSolver().updateB(grid, dt);
//
// Errors: every call that fails throws pica_gb300::Error (status + message);
// the C ABI itself never throws.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pica_gb300.h"

namespace pica_gb300 {

struct FP3 {
    double x = 0, y = 0, z = 0;
    FP3() = default;
    FP3(double a, double b, double c) : x(a), y(b), z(c) {}
    double norm2() const { return x * x + y * y + z * z; }
    double norm() const { return std::sqrt(norm2()); }
};
inline FP3 operator+(const FP3& a, const FP3& b) { return FP3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline FP3 operator-(const FP3& a, const FP3& b) { return FP3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline FP3 operator*(const FP3& a, double s) { return FP3(a.x * s, a.y * s, a.z * s); }
inline FP3 operator*(double s, const FP3& a) { return a * s; }
inline FP3 operator/(const FP3& a, double s) { return FP3(a.x / s, a.y / s, a.z / s); }
// Component-wise, as pica's Vector3 (math/Vectors.h).
inline FP3 operator*(const FP3& a, const FP3& b) { return FP3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline FP3 operator/(const FP3& a, const FP3& b) { return FP3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline bool operator==(const FP3& a, const FP3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
struct Int3 {
    int x = 0, y = 0, z = 0;
    Int3() = default;
    Int3(int a, int b, int c) : x(a), y(b), z(c) {}
};
inline bool operator==(const Int3& a, const Int3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Constants of pica math/Constants.h:9-18 (CGS, pi truncated as in pica), and the
// Constants<Real> accessors of Constants.h:23-34: each the namespace value cast to Real.
namespace constants {
const double pi = 3.14159265358;
const double c = 29979245800.0;
const double lightVelocity = c;
const double electronCharge = -4.80320427e-10;
const double electronMass = 9.10938215e-28;
const double protonMass = 1.672622964e-24;
const double planck = 1.0545716818e-27;
const double eV = 1.60217656535e-12;
const double meV = 1e6 * eV;
}  // namespace constants

template <typename Real>
struct Constants {
    static Real pi() { return static_cast<Real>(constants::pi); }
    static Real c() { return static_cast<Real>(constants::c); }
    static Real lightVelocity() { return static_cast<Real>(constants::lightVelocity); }
    static Real electronCharge() { return static_cast<Real>(constants::electronCharge); }
    static Real electronMass() { return static_cast<Real>(constants::electronMass); }
    static Real protonMass() { return static_cast<Real>(constants::protonMass); }
    static Real planck() { return static_cast<Real>(constants::planck); }
    static Real eV() { return static_cast<Real>(constants::eV); }
    static Real meV() { return static_cast<Real>(constants::meV); }
};

// One entry of pica's ParticleTypes table (particles/Particle.h:21-31).
struct ParticleType {
    double mass, charge;
};

// pica's global particle type table (particles/Particle.h:26-31).  Simulation fills
// it from Config::types; a host loop may set it itself before creating particles,
// as a pica host loop does.
namespace ParticleTypes {
inline std::vector<ParticleType> typesVector{{constants::electronMass, constants::electronCharge}};
inline const ParticleType* types = nullptr;   // nullptr: typesVector
inline int numTypes = 1;
inline const ParticleType& at(int i) { return types ? types[i] : typesVector[(size_t)i]; }
}  // namespace ParticleTypes

// Particle<Three> (particles/Particle.h:34-112): position, momentum stored
// normalised as p = P / (m c), weight factor and type index.  The fields are
// public; the accessors follow pica's: gamma = 1 / invGamma with invGamma =
// 1 / sqrt(1 + |p|^2), velocity p c invGamma, setVelocity p = v / sqrt(c^2 - |v|^2),
// mass and charge from the type table.
struct Particle3d {
    typedef FP3 PositionType;
    typedef FP3 MomentumType;
    typedef double GammaType, MassType, ChargeType, FactorType;
    typedef short TypeIndexType;

    FP3 position, p;
    double factor = 1.0;
    short typeIndex = 0;

    Particle3d() = default;
    Particle3d(const FP3& pos, const FP3& momentum, double f = 1, short type = 0)
        : position(pos), factor(f), typeIndex(type) {
        setMomentum(momentum);
    }
    FP3 getPosition() const { return position; }
    void setPosition(const FP3& v) { position = v; }
    FP3 getMomentum() const { return p * Constants<double>::c() * getMass(); }
    void setMomentum(const FP3& m) { p = m / (Constants<double>::c() * getMass()); }
    FP3 getP() const { return p; }
    void setP(const FP3& v) { p = v; }
    FP3 getVelocity() const { return p * (Constants<double>::c() * invGamma()); }
    void setVelocity(const FP3& v) { p = v / std::sqrt(constants::c * constants::c - v.norm2()); }
    double getGamma() const { return 1.0 / invGamma(); }
    double getMass() const { return ParticleTypes::at(typeIndex).mass; }
    double getCharge() const { return ParticleTypes::at(typeIndex).charge; }
    double getFactor() const { return factor; }
    void setFactor(double f) { factor = f; }
    short getType() const { return typeIndex; }
    void setType(short t) { typeIndex = t; }

private:
    double invGamma() const { return 1.0 / std::sqrt(1.0 + p.norm2()); }
};

// pica's ParticleArraySoA<Particle3d> (particles/ParticleArray.h:46-203): a host
// container of particles, one array per component (position, normalised momentum,
// factor, 1/gamma, type), whose elements are reached through ConstParticleRef /
// ParticleRef proxies with the accessors of Particle3d.  A host loop fills one and
// hands its particles to EnsembleSupercells::add.
class ParticleArraySoA {
public:
    typedef Particle3d Particle;

    class ConstParticleRef {
    public:
        ConstParticleRef(const ParticleArraySoA& a, int i) : a_(&a), i_(i) {}
        FP3 getPosition() const { return FP3(a_->x_[i_], a_->y_[i_], a_->z_[i_]); }
        FP3 getP() const { return FP3(a_->px_[i_], a_->py_[i_], a_->pz_[i_]); }
        FP3 getMomentum() const { return getP() * Constants<double>::c() * getMass(); }
        FP3 getVelocity() const { return getP() * Constants<double>::c() * a_->invGamma_[i_]; }
        double getGamma() const { return 1.0 / a_->invGamma_[i_]; }
        double getMass() const { return ParticleTypes::at(getType()).mass; }
        double getCharge() const { return ParticleTypes::at(getType()).charge; }
        double getFactor() const { return a_->factor_[i_]; }
        short getType() const { return a_->type_[i_]; }
        // The element as a Particle3d value.
        operator Particle3d() const {
            Particle3d q;
            q.position = getPosition();
            q.p = getP();
            q.factor = getFactor();
            q.typeIndex = getType();
            return q;
        }

    private:
        const ParticleArraySoA* a_;
        int i_;
    };

    class ParticleRef : public ConstParticleRef {
    public:
        ParticleRef(ParticleArraySoA& a, int i) : ConstParticleRef(a, i), m_(&a), j_(i) {}
        void setPosition(const FP3& r) { m_->x_[j_] = r.x; m_->y_[j_] = r.y; m_->z_[j_] = r.z; }
        void setP(const FP3& p) {
            m_->px_[j_] = p.x; m_->py_[j_] = p.y; m_->pz_[j_] = p.z;
            m_->invGamma_[j_] = 1.0 / std::sqrt(1.0 + p.norm2());
        }
        void setMomentum(const FP3& m) { setP(m / (Constants<double>::c() * this->getMass())); }
        void setVelocity(const FP3& v) { setP(v / std::sqrt(constants::c * constants::c - v.norm2())); }
        void setFactor(double f) { m_->factor_[j_] = f; }
        void setType(short t) { m_->type_[j_] = t; }

    private:
        ParticleArraySoA* m_;
        int j_;
    };

    int size() const { return (int)type_.size(); }
    ParticleRef operator[](int i) { return ParticleRef(*this, i); }
    ConstParticleRef operator[](int i) const { return ConstParticleRef(*this, i); }
    ParticleRef back() { return (*this)[size() - 1]; }
    ConstParticleRef back() const { return (*this)[size() - 1]; }
    void pushBack(const Particle3d& q) {
        x_.push_back(q.position.x); y_.push_back(q.position.y); z_.push_back(q.position.z);
        px_.push_back(q.p.x); py_.push_back(q.p.y); pz_.push_back(q.p.z);
        factor_.push_back(q.factor);
        invGamma_.push_back(1.0 / std::sqrt(1.0 + q.p.norm2()));
        type_.push_back(q.typeIndex);
    }
    void pushBack(const ConstParticleRef& r) { pushBack(static_cast<Particle3d>(r)); }
    void popBack() {
        for (auto* v : {&x_, &y_, &z_, &px_, &py_, &pz_, &factor_, &invGamma_}) v->pop_back();
        type_.pop_back();
    }

private:
    std::vector<double> x_, y_, z_, px_, py_, pz_, factor_, invGamma_;
    std::vector<short> type_;
};

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& msg) : std::runtime_error(msg), status(status) {}
    int status;
};

enum class Form { FP64Plain = PICA_FORM_FP64_PLAIN, FP32Cell = PICA_FORM_FP32_CELL };
enum class Shape { CIC = PICA_SHAPE_CIC, TSC = PICA_SHAPE_TSC };
enum class Depositor { Direct = PICA_DEPOSIT_DIRECT, Esirkepov = PICA_DEPOSIT_ESIRKEPOV };

struct Config {
    Int3 numCells{32, 32, 32};
    Int3 numCellsPerSupercell{2, 2, 2};
    FP3 step{1, 1, 1};
    double dt = 1;
    Form form = Form::FP64Plain;
    Shape shape = Shape::CIC;
    Depositor depositor = Depositor::Direct;
    std::vector<ParticleType> types{{constants::electronMass, constants::electronCharge}};
    double slack = 0.15;
    int resortEvery = 0;
};

class Simulation;
class YeeSolver;

// pica's Array3d (utility/Array.h:119-167): a 3D array with z fastest, index
// (i * ny + j) * nz + k, addressed by (i, j, k) or an Int3.
class Array3d {
public:
    Array3d() = default;
    explicit Array3d(const Int3& size) : n_(size), v_((size_t)size.x * size.y * size.z, 0.0) {}
    double& operator()(int i, int j, int k) { return v_[idx(i, j, k)]; }
    double operator()(int i, int j, int k) const { return v_[idx(i, j, k)]; }
    double& operator()(const Int3& n) { return v_[idx(n.x, n.y, n.z)]; }
    double operator()(const Int3& n) const { return v_[idx(n.x, n.y, n.z)]; }
    Int3 getSize() const { return n_; }
    size_t size() const { return v_.size(); }
    double* data() { return v_.data(); }
    const double* data() const { return v_.data(); }

private:
    size_t idx(int i, int j, int k) const { return ((size_t)i * n_.y + j) * n_.z + k; }
    Int3 n_;
    std::vector<double> v_;
};

// Host mirror of the device grid: pica's YeeGrid<Three> accessors (grid/YeeGrid.h:193-256,
// grid/Grid.h:13-83) on host arrays, moved to / from the device with upload() / download().
// The grid a Simulation owns is periodic with origin 0; a grid built with pica's
// constructor is a host container only (upload / download throw).
class YeeGrid {
public:
    YeeGrid() = default;
    YeeGrid(const FP3& origin, const FP3& step, const Int3& size) : n_(size), h_(step), o_(origin) {
        for (auto& a : f_) a = Array3d(size);
    }
#define PICA_GB300_COMPONENT(name, c)                                              \
    double& name(int i, int j, int k) { return f_[c](i, j, k); }                   \
    double name(int i, int j, int k) const { return f_[c](i, j, k); }              \
    double& name(const Int3& n) { return f_[c](n); }                               \
    double name(const Int3& n) const { return f_[c](n); }                          \
    Array3d& name() { return f_[c]; }                                              \
    const Array3d& name() const { return f_[c]; }
    PICA_GB300_COMPONENT(ex, 0)
    PICA_GB300_COMPONENT(ey, 1)
    PICA_GB300_COMPONENT(ez, 2)
    PICA_GB300_COMPONENT(bx, 3)
    PICA_GB300_COMPONENT(by, 4)
    PICA_GB300_COMPONENT(bz, 5)
    PICA_GB300_COMPONENT(jx, 6)
    PICA_GB300_COMPONENT(jy, 7)
    PICA_GB300_COMPONENT(jz, 8)
#undef PICA_GB300_COMPONENT
    Int3 getSize() const { return n_; }
    FP3 getStep() const { return h_; }
    FP3 getOrigin() const { return o_; }
    // Cell of a position: (position - origin) / step truncated toward zero (Grid.h:37).
    Int3 getCellIndex(const FP3& r) const {
        const FP3 q = (r - o_) / h_;
        return Int3((int)std::trunc(q.x), (int)std::trunc(q.y), (int)std::trunc(q.z));
    }
    // Offset of each component's node from the cell corner: pica's staggering (YeeGrid.h:11-14, 247-255).
    FP3 getShiftEx() const { return FP3(0, 0.5 * h_.y, 0.5 * h_.z); }
    FP3 getShiftEy() const { return FP3(0.5 * h_.x, 0, 0.5 * h_.z); }
    FP3 getShiftEz() const { return FP3(0.5 * h_.x, 0.5 * h_.y, 0); }
    FP3 getShiftBx() const { return FP3(0.5 * h_.x, 0, 0); }
    FP3 getShiftBy() const { return FP3(0, 0.5 * h_.y, 0); }
    FP3 getShiftBz() const { return FP3(0, 0, 0.5 * h_.z); }
    FP3 getShiftJx() const { return getShiftEx(); }
    FP3 getShiftJy() const { return getShiftEy(); }
    FP3 getShiftJz() const { return getShiftEz(); }
    inline void upload();
    inline void download();

private:
    friend class Simulation;
    friend class YeeSolver;
    pica_ctx* ctx_ = nullptr;
    Int3 n_;
    FP3 h_, o_;
    std::array<Array3d, 9> f_;
};

// Host staging of the device ensemble: add() collects particles, upload()
// routes them to supercells (EnsembleSupercells::add, EnsembleSupercells.h:41-45).
class EnsembleSupercells {
public:
    EnsembleSupercells() = default;
    // pica's constructor (EnsembleSupercells.h:25-34): a host-only container over
    // [minPosition, maxPosition) with numCells cells in supercells of numCellsPerSupercell
    // (add and getSupercellIndex work; upload and the device calls throw).  The
    // ensemble of a Simulation spans [0, numCells * step).
    EnsembleSupercells(const FP3& minPosition, const FP3& maxPosition, const Int3& numCells,
                       const Int3& numCellsPerSupercell)
        : S_(numCellsPerSupercell), min_(minPosition), max_(maxPosition), n_(numCells) {
        nsc_ = Int3((n_.x + S_.x - 1) / S_.x, (n_.y + S_.y - 1) / S_.y, (n_.z + S_.z - 1) / S_.z);
    }
    void add(const ParticleArraySoA::ConstParticleRef& r) { add(static_cast<Particle3d>(r)); }
    void add(const Particle3d& p) {
        x_.push_back(p.position.x); y_.push_back(p.position.y); z_.push_back(p.position.z);
        ux_.push_back(p.p.x); uy_.push_back(p.p.y); uz_.push_back(p.p.z);
        w_.push_back(p.factor); t_.push_back(p.typeIndex);
    }
    inline void upload();
    // All particles in ensemble order (type, supercell, slot).
    inline std::vector<Particle3d> particles() const;
    inline std::vector<int32_t> counts() const;
    Int3 getNumSupercells() const { return nsc_; }
    Int3 getNumCellsPerSupercell() const { return S_; }
    Int3 getNumCells() const { return n_; }
    FP3 getMinPosition() const { return min_; }
    FP3 getMaxPosition() const { return max_; }
    // pica's routing rule (EnsembleSupercells.h:54-57): floor((position - min) / supercell size),
    // supercell size = numCellsPerSupercell * (max - min) / numCells.
    Int3 getSupercellIndex(const Particle3d& p) const {
        const FP3 cell = (max_ - min_) / FP3(n_.x, n_.y, n_.z);
        const FP3 inv = FP3(1, 1, 1) / (FP3(S_.x, S_.y, S_.z) * cell);
        const FP3 q = (p.position - min_) * inv;
        return Int3((int)std::floor(q.x), (int)std::floor(q.y), (int)std::floor(q.z));
    }
    // The particles of one supercell (EnsembleSupercells.h:51-52), type by type in
    // slot order: a downloaded copy (the device holds the ensemble).
    inline std::vector<Particle3d> getParticles(const Int3& supercellIdx) const;
    // Number of particles on the device (pica's size() throws "not implemented").
    inline int64_t size() const;
    inline void migrate();
    // Sort every supercell by cell now (EnsembleOrdered::reorder, EnsembleOrdered.h:61-71).
    inline void reorder();

private:
    friend class Simulation;
    pica_ctx* ctx_ = nullptr;
    int ntypes_ = 1;
    Int3 nsc_, S_;
    FP3 min_, max_;
    Int3 n_;
    inline std::vector<Particle3d> download(std::vector<int32_t>* supercell) const;
    std::vector<double> x_, y_, z_, ux_, uy_, uz_, w_;
    std::vector<int32_t> t_;
};

inline void check(pica_ctx* ctx, int rc) {
    if (rc != PICA_OK) throw Error(rc, std::string(pica_status_string(rc)) + ": " + (ctx ? pica_last_error(ctx) : ""));
}

class Simulation {
public:
    explicit Simulation(const Config& c) {
        pica_config cfg{};
        cfg.n[0] = c.numCells.x; cfg.n[1] = c.numCells.y; cfg.n[2] = c.numCells.z;
        cfg.sc[0] = c.numCellsPerSupercell.x; cfg.sc[1] = c.numCellsPerSupercell.y; cfg.sc[2] = c.numCellsPerSupercell.z;
        cfg.h[0] = c.step.x; cfg.h[1] = c.step.y; cfg.h[2] = c.step.z;
        cfg.dt = c.dt;
        cfg.form = (int32_t)c.form; cfg.shape = (int32_t)c.shape; cfg.deposit = (int32_t)c.depositor;
        cfg.nspecies = (int32_t)c.types.size();
        for (size_t i = 0; i < c.types.size() && i < 4; i++) { cfg.mass[i] = c.types[i].mass; cfg.charge[i] = c.types[i].charge; }
        cfg.slack = c.slack;
        cfg.resort_every = c.resortEvery;
        check(nullptr, pica_ctx_create(&cfg, &ctx_));
        // The configured species become pica's global type table (Particle3d::getMass / getCharge).
        ParticleTypes::typesVector = c.types;
        ParticleTypes::types = nullptr;
        ParticleTypes::numTypes = (int)c.types.size();
        dt_ = c.dt;
        grid_.ctx_ = ctx_; grid_.n_ = c.numCells; grid_.h_ = c.step;
        for (auto& a : grid_.f_) a = Array3d(c.numCells);
        ens_.ctx_ = ctx_; ens_.ntypes_ = cfg.nspecies; ens_.S_ = c.numCellsPerSupercell;
        ens_.nsc_ = Int3(c.numCells.x / c.numCellsPerSupercell.x, c.numCells.y / c.numCellsPerSupercell.y,
                         c.numCells.z / c.numCellsPerSupercell.z);
        ens_.n_ = c.numCells;
        ens_.max_ = FP3(c.numCells.x * c.step.x, c.numCells.y * c.step.y, c.numCells.z * c.step.z);
    }
    ~Simulation() { if (ctx_) pica_ctx_destroy(ctx_); }
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    YeeGrid& grid() { return grid_; }
    EnsembleSupercells& ensemble() { return ens_; }
    pica_ctx* handle() { return ctx_; }
    double dt() const { return dt_; }
    void setStream(void* cudaStream) { check(ctx_, pica_set_stream(ctx_, cudaStream)); }
    // One full step: push + deposit, B(dt/2), E(dt), B(dt/2), migrate.
    void step(int n = 1) { check(ctx_, pica_step(ctx_, n)); }
    pica_diag diagnostics(double bgDensity = 0.0) {
        pica_diag d{};
        check(ctx_, pica_diagnostics(ctx_, bgDensity, &d));
        return d;
    }
    int64_t stepCount() { return pica_step_count(ctx_); }
    // Synthetic plasma generated on the device in place of ensemble().upload()
    // (FP32 cell form; see pica_generate_plasma).
    void generatePlasma(const std::vector<pica_plasma_spec>& specs) {
        check(ctx_, pica_generate_plasma(ctx_, specs.data(), (int32_t)specs.size()));
    }
    // Packed particle state of one species (used slots only; see pica_state_packed_slots):
    // statePackedSlots() lays the image out, copyStatePacked() moves one component of
    // it (host: pinned memory of statePackedSlots() x 4 or 8 bytes).
    int64_t statePackedSlots(int species = 0) {
        const int64_t n = pica_state_packed_slots(ctx_, species);
        if (n < 0) check(ctx_, (int)n);
        return n;
    }
    void copyStatePacked(int species, int comp, void* host, bool toDevice) {
        check(ctx_, pica_state_copy_packed(ctx_, species, comp, host, toDevice ? 1 : 0));
    }
    // The image part of supercells [scBegin, scEnd) (host: start of the whole image);
    // copyStream: the host copy on that cudaStream_t, the gather / scatter kernel on
    // the context stream (pica_state_copy_packed_range_on).
    void copyStatePackedRange(int species, int comp, void* host, bool toDevice, int scBegin, int scEnd,
                              void* copyStream = nullptr) {
        check(ctx_, pica_state_copy_packed_range_on(ctx_, species, comp, host, toDevice ? 1 : 0, scBegin, scEnd,
                                                    copyStream));
    }
    // The push in waitEvents.size() supercell ranges, range r after a wait for
    // waitEvents[r] (cudaEvent_t or nullptr); the rest of the step follows as in a
    // pica host loop: YeeSolver updateB(dt/2), updateE(dt), updateB(dt/2), ensemble().migrate().
    void pushDepositChunked(const std::vector<void*>& waitEvents) {
        check(ctx_, pica_push_deposit_chunked(ctx_, (int32_t)waitEvents.size(), waitEvents.data()));
    }
    // The same over supercell ranges [bounds[r], bounds[r+1]) of the caller's choice
    // (bounds.size() == waitEvents.size() + 1, from 0 to the supercell count).
    void pushDepositRanges(const std::vector<int32_t>& bounds, const std::vector<void*>& waitEvents) {
        if (bounds.size() != waitEvents.size() + 1) throw Error(PICA_ERR_INVALID, "one more bound than wait events");
        check(ctx_, pica_push_deposit_ranges(ctx_, (int32_t)waitEvents.size(), bounds.data(), waitEvents.data()));
    }
    // Complete state between steps; a Simulation of the same Config loaded from it
    // continues like this one (FP32 form: bit for bit).
    void saveCheckpoint(const std::string& path) { check(ctx_, pica_checkpoint_save(ctx_, path.c_str())); }
    void loadCheckpoint(const std::string& path) { check(ctx_, pica_checkpoint_load(ctx_, path.c_str())); }

private:
    pica_ctx* ctx_ = nullptr;
    double dt_ = 0;
    YeeGrid grid_;
    EnsembleSupercells ens_;
};

// Host loop around a Simulation (the PICADOR driver's role; periodic boundaries):
// run(n) steps in chunks, calls onDiagnostics every diagEvery steps and writes a
// checkpoint every checkpointEvery steps to checkpointPath + "<step>".
class Driver {
public:
    explicit Driver(Simulation& sim) : sim_(sim) {}
    int diagEvery = 0;
    int checkpointEvery = 0;
    std::string checkpointPath;
    double bgDensity = 0.0;
    std::function<void(int64_t, const pica_diag&)> onDiagnostics;

    void run(int64_t nsteps) {
        const int64_t end = sim_.stepCount() + nsteps;
        while (sim_.stepCount() < end) {
            const int64_t now = sim_.stepCount();
            int64_t target = end;
            if (diagEvery > 0) target = std::min(target, (now / diagEvery + 1) * diagEvery);
            if (checkpointEvery > 0) target = std::min(target, (now / checkpointEvery + 1) * checkpointEvery);
            sim_.step((int)(target - now));
            if (diagEvery > 0 && target % diagEvery == 0 && onDiagnostics) onDiagnostics(target, sim_.diagnostics(bgDensity));
            if (checkpointEvery > 0 && target % checkpointEvery == 0) sim_.saveCheckpoint(checkpointPath + std::to_string(target));
        }
    }

private:
    Simulation& sim_;
};

void YeeGrid::upload() {
    if (!ctx_) throw Error(PICA_ERR_INVALID, "this grid belongs to no Simulation");
    const double* p[9];
    for (int c = 0; c < 9; c++) p[c] = f_[c].data();
    check(ctx_, pica_upload_fields(ctx_, p));
}
void YeeGrid::download() {
    if (!ctx_) throw Error(PICA_ERR_INVALID, "this grid belongs to no Simulation");
    double* p[9];
    for (int c = 0; c < 9; c++) p[c] = f_[c].data();
    check(ctx_, pica_download_fields(ctx_, p));
}

void EnsembleSupercells::upload() {
    if (!ctx_) throw Error(PICA_ERR_INVALID, "this ensemble belongs to no Simulation");
    check(ctx_, pica_upload_particles(ctx_, (int64_t)w_.size(), x_.data(), y_.data(), z_.data(), ux_.data(),
                                      uy_.data(), uz_.data(), w_.data(), t_.data()));
    x_.clear(); y_.clear(); z_.clear(); ux_.clear(); uy_.clear(); uz_.clear(); w_.clear(); t_.clear();
}
std::vector<Particle3d> EnsembleSupercells::particles() const { return download(nullptr); }
std::vector<Particle3d> EnsembleSupercells::getParticles(const Int3& idx) const {
    std::vector<int32_t> s;
    const std::vector<Particle3d> all = download(&s);
    const int32_t want = (idx.x * nsc_.y + idx.y) * nsc_.z + idx.z;
    std::vector<Particle3d> out;
    for (size_t i = 0; i < all.size(); i++)
        if (s[i] == want) out.push_back(all[i]);
    return out;
}
int64_t EnsembleSupercells::size() const {
    if (!ctx_) throw Error(PICA_ERR_INVALID, "this ensemble belongs to no Simulation");
    const int64_t n = pica_num_particles(ctx_);
    if (n < 0) check(ctx_, (int)n);
    return n;
}
std::vector<Particle3d> EnsembleSupercells::download(std::vector<int32_t>* supercell) const {
    if (!ctx_) throw Error(PICA_ERR_INVALID, "this ensemble belongs to no Simulation");
    const int64_t n = pica_num_particles(ctx_);
    if (n < 0) check(ctx_, (int)n);
    std::vector<double> a[7];
    for (auto& v : a) v.resize(n);
    std::vector<int32_t> t(n), s(n);
    check(ctx_, pica_download_particles(ctx_, a[0].data(), a[1].data(), a[2].data(), a[3].data(), a[4].data(),
                                        a[5].data(), a[6].data(), t.data(), s.data()));
    std::vector<Particle3d> out(n);
    for (int64_t i = 0; i < n; i++) {
        out[i].position = FP3(a[0][i], a[1][i], a[2][i]);
        out[i].p = FP3(a[3][i], a[4][i], a[5][i]);
        out[i].factor = a[6][i];
        out[i].typeIndex = (short)t[i];
    }
    if (supercell) *supercell = std::move(s);
    return out;
}
std::vector<int32_t> EnsembleSupercells::counts() const {
    std::vector<int32_t> c((size_t)ntypes_ * nsc_.x * nsc_.y * nsc_.z);
    check(ctx_, pica_get_counts(ctx_, c.data()));
    return c;
}
void EnsembleSupercells::migrate() { check(ctx_, pica_migrate(ctx_)); }
void EnsembleSupercells::reorder() { check(ctx_, pica_reorder(ctx_)); }

// pica YeeSolver (fieldSolver/YeeSolver.h:11-38) on the periodic device grid.
class YeeSolver {
public:
    void updateE(YeeGrid& g, double dt) { check(g.ctx_, pica_update_e(g.ctx_, dt)); }
    void updateB(YeeGrid& g, double dt) { check(g.ctx_, pica_update_b(g.ctx_, dt)); }
};

// FieldInterpolator::get + BorisPusher::push + CurrentDepositor::deposit for
// every particle of every supercell (the supercell loop of a pica host loop).
inline void pushSupercells(Simulation& sim) { check(sim.handle(), pica_push_deposit(sim.handle())); }

}  // namespace pica_gb300
