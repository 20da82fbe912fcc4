// pica_gb300.hpp -- header-only C++ mirror of pica's hot-path classes over the
// pica_gb300 C ABI (pica_gb300.h).
//
// pica's host loop constructs a YeeGrid, an EnsembleSupercells of
// ParticleArraySoA<Particle3d>, a BorisPusher, and per supercell a
// FieldInterpolatorCICSupercell and a CurrentDepositorCICSupercell, then calls
// get / push / deposit per particle and YeeSolver::updateB/updateE per step.
// This header keeps those type names, template parameters and constructors.
// The grid and the ensemble are host containers that bind to one device
// context the first time an operator acts on them; the per-particle inner loop
// becomes one bulk call:
//
//   pica:                                             pica_gb300 (this header):
//   #include "pica/..."                               #include "pica_gb300.hpp"
//   using namespace pica;                             using namespace pica_gb300;
//   YeeGrid<Three, double> grid(origin, step, size);  (same)
//   EnsembleSupercells<ParticleArraySoA<Particle3d>>  (same)
//       ens(min, max, numCells, numCellsPerSupercell);
//   ens.add(particle);                                (same)
//   BorisPusher<Particle3d, double> pusher(dt);        (same)
//   FieldInterpolatorCICSupercell<double> fi(grid, min, S);   (same)
//   CurrentDepositorCICSupercell<double> cd(grid, min, S);    (same)
//   for each supercell, particle:                     pushSupercells(ens, fi, pusher, cd);
//       fi.get(...); pusher.push(...); cd.deposit(...);
//   YeeSolver solver; solver.updateB(grid, dt / 2);   (same)
//   grid.ex(i, j, k), ens.getParticles(idx)           (same: read back from the device on demand)
//
// Host and device copies are kept in step by the library: element writes and
// added particles go to the device before the next operator; after an operator
// the next host read fetches the device state (one copy of all arrays).  The
// device grid is periodic over the ensemble's domain [min, max) with no guard
// layers, so the grid's size must equal the ensemble's numCells; the supercell
// migration that a pica host loop writes by hand happens inside the library
// before the next push or read.  double operators run the FP64 plain form
// (pica's own arithmetic), float operators the FP32 cell form.
//
// The explicit form of the same API (Simulation with a Config, explicit
// upload / download / migrate) is below as well.
//
// Errors: every call that fails throws pica_gb300::Error (status + message);
// the C ABI itself never throws.  There is no CPU implementation of any
// operator: without a GPU, binding a context throws.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
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

// pica's Dimension (math/Dimension.h): only Three has device operators here.
enum Dimension { One = 1, Two = 2, Three = 3 };

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

// pica's global particle type table (particles/Particle.h:26-31).  A host loop
// fills it before creating particles, as a pica host loop does; Simulation fills
// it from Config::types.  The device context takes its species from it.
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

template <class PA>
class EnsembleSupercells;

// pica's ParticleArraySoA<ParticleType> (particles/ParticleArray.h:46-203): a host
// container of particles, one array per component (position, normalised momentum,
// factor, 1/gamma, type), whose elements are reached through ConstParticleRef /
// ParticleRef proxies with the accessors of Particle3d.  The device ensemble holds
// 3D particles, so ParticleType is Particle3d.  An array that an ensemble hands
// out (getParticles) reports writes through its references to that ensemble,
// which sends them to the device before the next operator.
template <class ParticleType>
class ParticleArraySoA {
    static_assert(std::is_same<ParticleType, Particle3d>::value, "the device ensemble holds Particle3d particles");

public:
    typedef ParticleType Particle;

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
        void setPosition(const FP3& r) { m_->x_[j_] = r.x; m_->y_[j_] = r.y; m_->z_[j_] = r.z; m_->touch(); }
        void setP(const FP3& p) {
            m_->px_[j_] = p.x; m_->py_[j_] = p.y; m_->pz_[j_] = p.z;
            m_->invGamma_[j_] = 1.0 / std::sqrt(1.0 + p.norm2());
            m_->touch();
        }
        void setMomentum(const FP3& m) { setP(m / (Constants<double>::c() * this->getMass())); }
        void setVelocity(const FP3& v) { setP(v / std::sqrt(constants::c * constants::c - v.norm2())); }
        void setFactor(double f) { m_->factor_[j_] = f; m_->touch(); }
        void setType(short t) { m_->type_[j_] = t; m_->touch(); }

    private:
        ParticleArraySoA* m_;
        int j_;
    };

    ParticleArraySoA() = default;
    // A copy is a plain host array: it reports to no ensemble.
    ParticleArraySoA(const ParticleArraySoA& o)
        : x_(o.x_), y_(o.y_), z_(o.z_), px_(o.px_), py_(o.py_), pz_(o.pz_), factor_(o.factor_),
          invGamma_(o.invGamma_), type_(o.type_) {}
    ParticleArraySoA& operator=(const ParticleArraySoA& o) {
        x_ = o.x_; y_ = o.y_; z_ = o.z_; px_ = o.px_; py_ = o.py_; pz_ = o.pz_;
        factor_ = o.factor_; invGamma_ = o.invGamma_; type_ = o.type_;
        touch();
        return *this;
    }

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
        touch();
    }
    void pushBack(const ConstParticleRef& r) { pushBack(static_cast<Particle3d>(r)); }
    void popBack() {
        for (auto* v : {&x_, &y_, &z_, &px_, &py_, &pz_, &factor_, &invGamma_}) v->pop_back();
        type_.pop_back();
        touch();
    }

private:
    template <class PA>
    friend class EnsembleSupercells;
    void touch() { if (owner_) *owner_ = true; }
    bool* owner_ = nullptr;   // the "host copy changed" flag of the ensemble that handed this array out
    std::vector<double> x_, y_, z_, px_, py_, pz_, factor_, invGamma_;
    std::vector<short> type_;
};

// pica's ParticleArray<Particle, representation>::Type (particles/ParticleArray.h:217-231);
// the device ensemble is structure-of-arrays only.
enum ParticleRepresentation { ParticleRepresentation_AoS, ParticleRepresentation_SoA };
template <class Particle, ParticleRepresentation storage>
struct ParticleArray;
template <class Particle>
struct ParticleArray<Particle, ParticleRepresentation_SoA> {
    typedef ParticleArraySoA<Particle> Type;
};

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& msg) : std::runtime_error(msg), status(status) {}
    int status;
};

inline void check(pica_ctx* ctx, int rc) {
    if (rc != PICA_OK) throw Error(rc, std::string(pica_status_string(rc)) + ": " + (ctx ? pica_last_error(ctx) : ""));
}

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

// pica's Array3d<T> (utility/Array.h:119-167): a 3D array with z fastest, index
// (i * ny + j) * nz + k, addressed by (i, j, k) or an Int3.
template <typename T>
class Array3d {
public:
    typedef T ValueType;
    Array3d() = default;
    explicit Array3d(const Int3& size) : n_(size), v_((size_t)size.x * size.y * size.z, T(0)) {}
    T& operator()(int i, int j, int k) { return v_[idx(i, j, k)]; }
    T operator()(int i, int j, int k) const { return v_[idx(i, j, k)]; }
    T& operator()(const Int3& n) { return v_[idx(n.x, n.y, n.z)]; }
    T operator()(const Int3& n) const { return v_[idx(n.x, n.y, n.z)]; }
    Int3 getSize() const { return n_; }
    size_t size() const { return v_.size(); }
    T* data() { return v_.data(); }
    const T* data() const { return v_.data(); }

private:
    size_t idx(int i, int j, int k) const { return ((size_t)i * n_.y + j) * n_.z + k; }
    Int3 n_;
    std::vector<T> v_;
};

namespace detail {
// One device context shared by a grid and an ensemble, and what its host copies
// know of it.
struct Binding {
    pica_ctx* ctx = nullptr;
    pica_config cfg{};
    bool fieldsStale = false;     // the device changed the fields since the grid's host copy was read
    bool pending = false;         // a push awaits its migration
    uint64_t particleEpoch = 1;   // bumped by every call that changes the device particles
    Binding() = default;
    Binding(const Binding&) = delete;
    Binding& operator=(const Binding&) = delete;
    ~Binding() { if (ctx) pica_ctx_destroy(ctx); }
    // The migration of the last push, before anything reads or replaces the ensemble.
    void settle() {
        if (pending) {
            pending = false;
            check(ctx, pica_migrate(ctx));
            particleEpoch++;
        }
    }
};
inline bool sameConfig(const pica_config& a, const pica_config& b) {
    for (int d = 0; d < 3; d++)
        if (a.n[d] != b.n[d] || a.sc[d] != b.sc[d] || a.h[d] != b.h[d]) return false;
    if (a.dt != b.dt || a.form != b.form || a.shape != b.shape || a.deposit != b.deposit || a.nspecies != b.nspecies ||
        a.slack != b.slack || a.resort_every != b.resort_every || a.threads != b.threads)
        return false;
    for (int q = 0; q < a.nspecies; q++)
        if (a.mass[q] != b.mass[q] || a.charge[q] != b.charge[q]) return false;
    return true;
}
struct Access;
}  // namespace detail

// pica's YeeGrid<Dimension, Real> (grid/YeeGrid.h:193-256, grid/Grid.h:13-83).  The
// device operators work on YeeGrid<Three, Real>.
template <Dimension D, typename Real = double>
class YeeGrid;

// Host copy of the grid with pica's accessors.  Once bound to a device context
// (by pushSupercells, a YeeSolver update or a Simulation), element writes reach
// the device before the next operator, and the first read after an operator
// fetches the device fields (all nine arrays, once).
template <typename Real>
class YeeGrid<Three, Real> {
public:
    typedef Int3 IndexType;
    typedef FP3 PositionType;
    typedef Real ValueType;
    typedef Array3d<Real> ArrayType;

    YeeGrid(const FP3& origin, const FP3& step, const Int3& size) : n_(size), h_(step), o_(origin) {
        for (auto& a : f_) a = ArrayType(size);
    }
    YeeGrid(const YeeGrid&) = delete;
    YeeGrid& operator=(const YeeGrid&) = delete;
#define PICA_GB300_COMPONENT(name, c)                                                      \
    Real& name(int i, int j, int k) { write(); return f_[c](i, j, k); }                    \
    Real name(int i, int j, int k) const { read(); return f_[c](i, j, k); }                \
    Real& name(const Int3& n) { write(); return f_[c](n); }                                \
    Real name(const Int3& n) const { read(); return f_[c](n); }                            \
    ArrayType& name() { write(); return f_[c]; }                                           \
    const ArrayType& name() const { read(); return f_[c]; }
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
    // Explicit copies (bound grids only; PICA_ERR_INVALID before the grid is bound).
    void upload() { need(); push(); }
    void download() { need(); pull(); }

private:
    friend struct detail::Access;
    void need() const {
        if (!b_) throw Error(PICA_ERR_INVALID, "this grid is bound to no device context yet");
    }
    void read() const {
        if (b_ && b_->fieldsStale && !dirty_) const_cast<YeeGrid*>(this)->pull();
    }
    void write() {
        read();
        dirty_ = true;
    }
    void pull() {
        std::array<std::vector<double>, 9> t;
        double* p[9];
        for (int c = 0; c < 9; c++) {
            if (std::is_same<Real, double>::value) {
                p[c] = reinterpret_cast<double*>(f_[c].data());
            } else {
                t[c].resize(f_[c].size());
                p[c] = t[c].data();
            }
        }
        check(b_->ctx, pica_download_fields(b_->ctx, p));
        if (!std::is_same<Real, double>::value)
            for (int c = 0; c < 9; c++) std::copy(t[c].begin(), t[c].end(), f_[c].data());
        b_->fieldsStale = false;
        dirty_ = false;
    }
    void push() {
        std::array<std::vector<double>, 9> t;
        const double* p[9];
        for (int c = 0; c < 9; c++) {
            if (std::is_same<Real, double>::value) {
                p[c] = reinterpret_cast<const double*>(f_[c].data());
            } else {
                t[c].assign(f_[c].data(), f_[c].data() + f_[c].size());
                p[c] = t[c].data();
            }
        }
        check(b_->ctx, pica_upload_fields(b_->ctx, p));
        b_->fieldsStale = false;
        dirty_ = false;
    }
    void flush() {
        if (dirty_) push();
    }
    std::shared_ptr<detail::Binding> b_;
    bool dirty_ = false;   // the host copy changed since the device received it
    Int3 n_;
    FP3 h_, o_;
    std::array<ArrayType, 9> f_;
};

// pica's EnsembleSupercells<ParticleArray> (particles/EnsembleSupercells.h:15-69):
// particles routed to supercells of numCellsPerSupercell cells over [min, max)
// by floor((position - min) / supercellSize).  The host copy keeps one
// ParticleArray per supercell (its particles type by type); once bound to a
// device context, added or modified particles reach the device before the next
// operator, and the first read after an operator fetches the device ensemble.
// Positions outside [min, max) wrap periodically on the device.
template <class PA>
class EnsembleSupercells {
public:
    typedef PA ParticleArray;
    typedef typename PA::Particle Particle;
    typedef typename PA::ParticleRef ParticleRef;
    typedef typename PA::ConstParticleRef ConstParticleRef;
    typedef FP3 PositionType;
    typedef Int3 IndexType;

    // pica's constructor (EnsembleSupercells.h:25-34).
    EnsembleSupercells(const FP3& minPosition, const FP3& maxPosition, const Int3& numCells,
                       const Int3& numCellsPerSupercell)
        : S_(numCellsPerSupercell), min_(minPosition), max_(maxPosition), n_(numCells) {
        nsc_ = Int3((n_.x + S_.x - 1) / S_.x, (n_.y + S_.y - 1) / S_.y, (n_.z + S_.z - 1) / S_.z);
        cells_.resize((size_t)nsc_.x * nsc_.y * nsc_.z);
        own();
    }
    EnsembleSupercells(const EnsembleSupercells&) = delete;
    EnsembleSupercells& operator=(const EnsembleSupercells&) = delete;

    // EnsembleSupercells::add (EnsembleSupercells.h:41-45): a Particle3d or a reference.
    template <class P>
    void add(const P& particle) {
        const Particle3d q = static_cast<Particle3d>(particle);
        ensureHost();
        cells_[linear(wrapped(getSupercellIndex(q)))].pushBack(q);
    }
    // The particles of one supercell (EnsembleSupercells.h:49-52), type by type.
    PA& getParticles(const Int3& idx) {
        ensureHost();
        return cells_[linear(idx)];
    }
    const PA& getParticles(const Int3& idx) const {
        ensureHost();
        return cells_[linear(idx)];
    }
    Int3 getNumSupercells() const { return nsc_; }
    Int3 getNumCellsPerSupercell() const { return S_; }
    Int3 getNumCells() const { return n_; }
    FP3 getMinPosition() const { return min_; }
    FP3 getMaxPosition() const { return max_; }
    // pica's routing rule (EnsembleSupercells.h:54-57): floor((position - min) / supercell size),
    // supercell size = numCellsPerSupercell * (max - min) / numCells.
    template <class P>
    Int3 getSupercellIndex(const P& particle) const {
        const Particle3d p = static_cast<Particle3d>(particle);
        const FP3 cell = (max_ - min_) / FP3(n_.x, n_.y, n_.z);
        const FP3 inv = FP3(1, 1, 1) / (FP3(S_.x, S_.y, S_.z) * cell);
        const FP3 q = (p.position - min_) * inv;
        return Int3((int)std::floor(q.x), (int)std::floor(q.y), (int)std::floor(q.z));
    }
    // Number of particles (pica's size() throws "not implemented").
    int64_t size() const {
        if (b_ && !dirty_) {
            const int64_t n = pica_num_particles(b_->ctx);
            if (n < 0) check(b_->ctx, (int)n);
            return n;
        }
        int64_t n = 0;
        for (auto& a : cells_) n += a.size();
        return n;
    }
    // All particles in ensemble order (type, supercell, slot) and the per-supercell
    // counts (counts[type * supercells + s]), read from the device.
    inline std::vector<Particle3d> particles() const;
    inline std::vector<int32_t> counts() const;
    // Explicit calls of the Simulation form: send the host copy now; finish the
    // push's migration now; sort every supercell by cell now
    // (EnsembleOrdered::reorder, EnsembleOrdered.h:61-71).
    void upload() { need(); flush(true); }
    void migrate() {
        need();
        b_->pending = false;
        check(b_->ctx, pica_migrate(b_->ctx));
        b_->particleEpoch++;
    }
    void reorder() {
        need();
        b_->settle();
        flush(false);
        check(b_->ctx, pica_reorder(b_->ctx));
        b_->particleEpoch++;
    }
    // In-supercell sort by cell every resortEvery steps on the device (-1: 0 for
    // double operators, 2 for float operators).  Read when the ensemble is bound.
    int resortEvery = -1;

private:
    friend struct detail::Access;
    void need() const {
        if (!b_) throw Error(PICA_ERR_INVALID, "this ensemble is bound to no device context yet");
    }
    size_t linear(const Int3& i) const { return ((size_t)i.x * nsc_.y + i.y) * nsc_.z + i.z; }
    Int3 wrapped(const Int3& i) const {
        auto w = [](int a, int n) { a %= n; return a < 0 ? a + n : a; };
        return Int3(w(i.x, nsc_.x), w(i.y, nsc_.y), w(i.z, nsc_.z));
    }
    void own() {
        for (auto& a : cells_) a.owner_ = &dirty_;
    }
    inline std::vector<Particle3d> download(std::vector<int32_t>* supercell) const;
    // Bring the host copy up to date (after a device operator).
    void ensureHost() const {
        if (b_ && !dirty_ && epoch_ != b_->particleEpoch) const_cast<EnsembleSupercells*>(this)->pull();
    }
    void pull() {
        std::vector<int32_t> s;
        const std::vector<Particle3d> all = download(&s);
        for (auto& a : cells_) a = PA();
        for (size_t i = 0; i < all.size(); i++) cells_[(size_t)s[i]].pushBack(all[i]);
        own();
        dirty_ = false;
        epoch_ = b_->particleEpoch;
    }
    // Send the host copy to the device if it changed (or always).
    void flush(bool always) {
        if (!dirty_ && !always) return;
        b_->settle();
        int64_t n = 0;
        for (auto& a : cells_) n += a.size();
        std::vector<double> v[7];
        for (auto& x : v) x.reserve((size_t)n);
        std::vector<int32_t> t;
        t.reserve((size_t)n);
        for (auto& a : cells_)
            for (int i = 0; i < a.size(); i++) {
                const Particle3d q = static_cast<Particle3d>(a[i]);
                v[0].push_back(q.position.x - min_.x); v[1].push_back(q.position.y - min_.y);
                v[2].push_back(q.position.z - min_.z);
                v[3].push_back(q.p.x); v[4].push_back(q.p.y); v[5].push_back(q.p.z);
                v[6].push_back(q.factor);
                t.push_back(q.typeIndex);
            }
        check(b_->ctx, pica_upload_particles(b_->ctx, n, v[0].data(), v[1].data(), v[2].data(), v[3].data(),
                                             v[4].data(), v[5].data(), v[6].data(), t.data()));
        dirty_ = false;
        b_->particleEpoch++;   // the device holds them in its own order now
    }
    std::shared_ptr<detail::Binding> b_;
    Int3 nsc_, S_;
    FP3 min_, max_;
    Int3 n_;
    mutable std::vector<PA> cells_;   // host copy: one array per supercell
    mutable bool dirty_ = true;       // the host copy changed since the device received it
    mutable uint64_t epoch_ = 0;      // the binding's particle epoch the host copy reflects
};

// pica's EnsembleUnordered (particles/EnsembleUnordered.h:14-40): one flat host
// array of particles in insertion order.  A flat array on the device is pushed
// through pica_push_flat (include/pica_gb300.h).
template <class PA>
class EnsembleUnordered {
public:
    typedef PA ParticleArray;
    typedef typename PA::Particle Particle;
    typedef typename PA::ParticleRef ParticleRef;
    typedef typename PA::ConstParticleRef ConstParticleRef;
    typedef FP3 PositionType;

    EnsembleUnordered(const FP3& minPosition, const FP3& maxPosition) : min_(minPosition), max_(maxPosition) {}
    FP3 getMinPosition() const { return min_; }
    FP3 getMaxPosition() const { return max_; }
    int size() const { return particles_.size(); }
    template <class P>
    void add(const P& particle) { particles_.pushBack(static_cast<Particle3d>(particle)); }
    PA& getParticles() { return particles_; }
    const PA& getParticles() const { return particles_; }

protected:
    PA particles_;
    FP3 min_, max_;
};

// pica's EnsembleOrdered (particles/EnsembleOrdered.h:17-71): reorder() sorts the
// array lexicographically by position, on the device (pica_order_by_position_host),
// stably: ties keep their order, where pica's std::sort leaves it unspecified.
template <class PA>
class EnsembleOrdered : public EnsembleUnordered<PA> {
public:
    EnsembleOrdered(const FP3& minPosition, const FP3& maxPosition) : EnsembleUnordered<PA>(minPosition, maxPosition) {}
    void reorder() {
        const PA& a = this->particles_;
        const int n = a.size();
        std::vector<double> x((size_t)n), y((size_t)n), z((size_t)n);
        for (int i = 0; i < n; i++) {
            const FP3 r = a[i].getPosition();
            x[(size_t)i] = r.x; y[(size_t)i] = r.y; z[(size_t)i] = r.z;
        }
        std::vector<int64_t> order((size_t)n);
        check(nullptr, pica_order_by_position_host(n, 3, x.data(), y.data(), z.data(), order.data()));
        PA sorted;
        for (int i = 0; i < n; i++) sorted.pushBack(a[(int)order[(size_t)i]]);
        this->particles_ = sorted;
    }
};

// pica's representation selector (particles/Ensemble.h:20-53).
enum EnsembleRepresentation {
    EnsembleRepresentation_Unordered,
    EnsembleRepresentation_Ordered,
    EnsembleRepresentation_Supercells
};
template <class PA, EnsembleRepresentation storage>
struct Ensemble;
template <class PA>
struct Ensemble<PA, EnsembleRepresentation_Unordered> {
    typedef EnsembleUnordered<PA> Type;
};
template <class PA>
struct Ensemble<PA, EnsembleRepresentation_Ordered> {
    typedef EnsembleOrdered<PA> Type;
};
template <class PA>
struct Ensemble<PA, EnsembleRepresentation_Supercells> {
    typedef EnsembleSupercells<PA> Type;
};

// ---------------------------------------------------------------------------
// Operators.  Each carries the configuration of the bulk call that replaces its
// per-particle method (no per-particle get / push / deposit: they would run on
// the CPU, and there is no CPU path).
// ---------------------------------------------------------------------------

// pica's BorisPusher<Particle, Real> (particlePush/BorisPusher.h:13-30): dt and the
// per-type coefficients q dt / (2 m c) from the ParticleTypes table.
template <class Particle, typename Real>
struct BorisPusher {
    std::vector<Real> coeffVector;
    Real* coeff;
    Real dt;
    explicit BorisPusher(Real dt) : dt(dt) {
        coeffVector.resize((size_t)ParticleTypes::numTypes);
        coeff = coeffVector.data();
        for (int i = 0; i < ParticleTypes::numTypes; i++)
            coeff[i] = static_cast<Real>(ParticleTypes::at(i).charge * dt /
                                         (2.0 * ParticleTypes::at(i).mass * Constants<double>::c()));
    }
};

#define PICA_GB300_INTERPOLATOR(Name, SHAPE)                                                         \
    template <class GridType>                                                                        \
    class Name;                                                                                      \
    template <typename Real>                                                                         \
    class Name<YeeGrid<Three, Real>> {                                                               \
    public:                                                                                          \
        typedef YeeGrid<Three, Real> GridType;                                                       \
        typedef Real RealType;                                                                       \
        static constexpr int shape = SHAPE;                                                          \
        explicit Name(const GridType& g) : grid(g) {}                                                \
        const GridType& grid;                                                                        \
    };                                                                                               \
    template <typename Real>                                                                         \
    class Name##Supercell {                                                                          \
    public:                                                                                          \
        typedef YeeGrid<Three, Real> GridType;                                                       \
        typedef Real RealType;                                                                       \
        static constexpr int shape = SHAPE;                                                          \
        Name##Supercell(const GridType& g, const FP3& minPos, const Int3& cellsPerSupercell)          \
            : grid(g), minPosition(minPos), numCellsPerSupercell(cellsPerSupercell) {}               \
        const GridType& grid;                                                                        \
        FP3 minPosition;                                                                             \
        Int3 numCellsPerSupercell;                                                                   \
    };
// pica's FieldInterpolatorCIC<YeeGrid<Three, Real>> and FieldInterpolatorCICSupercell<Real>
// (fieldInterpolation/FieldInterpolatorYeeGrid.h:137-187, 188-283), and their TSC
// siblings (quadratic B-spline form factor; no counterpart in pica).
PICA_GB300_INTERPOLATOR(FieldInterpolatorCIC, PICA_SHAPE_CIC)
PICA_GB300_INTERPOLATOR(FieldInterpolatorTSC, PICA_SHAPE_TSC)
#undef PICA_GB300_INTERPOLATOR

#define PICA_GB300_DEPOSITOR(Name, SHAPE, KIND)                                                      \
    template <class GridType>                                                                        \
    class Name;                                                                                      \
    template <typename Real>                                                                         \
    class Name<YeeGrid<Three, Real>> {                                                               \
    public:                                                                                          \
        typedef YeeGrid<Three, Real> GridType;                                                       \
        typedef Real RealType;                                                                       \
        static constexpr int shape = SHAPE;                                                          \
        static constexpr int deposit = KIND;                                                         \
        explicit Name(GridType& g) : grid(g) {}                                                      \
        GridType& grid;                                                                              \
    };                                                                                               \
    template <typename Real>                                                                         \
    class Name##Supercell {                                                                          \
    public:                                                                                          \
        typedef YeeGrid<Three, Real> GridType;                                                       \
        typedef Real RealType;                                                                       \
        static constexpr int shape = SHAPE;                                                          \
        static constexpr int deposit = KIND;                                                         \
        Name##Supercell(GridType& g, const FP3& minPos, const Int3& cellsPerSupercell)                \
            : grid(g), minPosition(minPos), numCellsPerSupercell(cellsPerSupercell) {}               \
        GridType& grid;                                                                              \
        FP3 minPosition;                                                                             \
        Int3 numCellsPerSupercell;                                                                   \
    };
// pica's CurrentDepositorCIC<YeeGrid<Three, Real>> and CurrentDepositorCICSupercell<Real>
// (currentDeposition/CurrentDepositorYeeGrid.h:126-163, 169-264): direct deposition of
// q w v at the new position.  The TSC siblings deposit directly with the TSC form
// factor, and the Esirkepov depositors conserve charge exactly (T. Zh. Esirkepov,
// Comput. Phys. Commun. 135 (2001) 144) with the interpolator's form factor; pica has
// neither.
PICA_GB300_DEPOSITOR(CurrentDepositorCIC, PICA_SHAPE_CIC, PICA_DEPOSIT_DIRECT)
PICA_GB300_DEPOSITOR(CurrentDepositorTSC, PICA_SHAPE_TSC, PICA_DEPOSIT_DIRECT)
PICA_GB300_DEPOSITOR(CurrentDepositorEsirkepov, 0, PICA_DEPOSIT_ESIRKEPOV)
#undef PICA_GB300_DEPOSITOR

namespace detail {
struct Access {
    template <typename Real, class PA>
    static void attach(YeeGrid<Three, Real>& g, EnsembleSupercells<PA>& e, const std::shared_ptr<Binding>& b) {
        g.b_ = b;
        g.dirty_ = false;
        e.b_ = b;
        e.dirty_ = false;
        e.epoch_ = b->particleEpoch;
    }
    template <typename Real>
    static void flush(YeeGrid<Three, Real>& g) { g.flush(); }
    template <class PA>
    static void flush(EnsembleSupercells<PA>& e) { e.flush(false); }
    template <class PA>
    static void replaced(EnsembleSupercells<PA>& e) { e.dirty_ = false; }

    static pica_config base(const Int3& n, const FP3& h, double dt, bool fp64) {
        pica_config cfg{};
        cfg.n[0] = n.x; cfg.n[1] = n.y; cfg.n[2] = n.z;
        cfg.h[0] = h.x; cfg.h[1] = h.y; cfg.h[2] = h.z;
        cfg.dt = dt;
        cfg.form = fp64 ? PICA_FORM_FP64_PLAIN : PICA_FORM_FP32_CELL;
        if (ParticleTypes::numTypes < 1 || ParticleTypes::numTypes > 4)
            throw Error(PICA_ERR_INVALID, "the ParticleTypes table must hold 1 to 4 types");
        cfg.nspecies = ParticleTypes::numTypes;
        for (int q = 0; q < cfg.nspecies; q++) {
            cfg.mass[q] = ParticleTypes::at(q).mass;
            cfg.charge[q] = ParticleTypes::at(q).charge;
        }
        cfg.slack = 0.15;
        return cfg;
    }
    // The configuration of a bulk push over (grid, ensemble).
    template <typename Real, class PA>
    static pica_config configFor(const YeeGrid<Three, Real>& g, const EnsembleSupercells<PA>& e, double dt, int shape,
                                 int deposit) {
        if (!(g.n_ == e.n_))
            throw Error(PICA_ERR_INVALID, "the grid's size must equal the ensemble's numCells (the device grid is "
                                          "periodic over the ensemble's domain, with no guard layers)");
        const FP3 cell = (e.max_ - e.min_) / FP3(e.n_.x, e.n_.y, e.n_.z);
        if (std::fabs(cell.x - g.h_.x) > 1e-9 * g.h_.x || std::fabs(cell.y - g.h_.y) > 1e-9 * g.h_.y ||
            std::fabs(cell.z - g.h_.z) > 1e-9 * g.h_.z)
            throw Error(PICA_ERR_INVALID, "the grid's step differs from the ensemble's cell size");
        const bool fp64 = std::is_same<Real, double>::value;
        pica_config cfg = base(g.n_, g.h_, dt, fp64);
        cfg.sc[0] = e.S_.x; cfg.sc[1] = e.S_.y; cfg.sc[2] = e.S_.z;
        cfg.shape = shape;
        cfg.deposit = deposit;
        cfg.resort_every = e.resortEvery >= 0 ? e.resortEvery : (fp64 ? 0 : 2);
        return cfg;
    }
    static std::shared_ptr<Binding> make(const pica_config& cfg) {
        auto b = std::make_shared<Binding>();
        b->cfg = cfg;
        check(nullptr, pica_ctx_create(&cfg, &b->ctx));
        return b;
    }
    // A context of the grid alone (a field solve before any push): one-cell supercells.
    template <typename Real>
    static void bindFields(YeeGrid<Three, Real>& g) {
        pica_config cfg = base(g.n_, g.h_, 1.0, std::is_same<Real, double>::value);
        cfg.sc[0] = cfg.sc[1] = cfg.sc[2] = 1;
        cfg.shape = PICA_SHAPE_CIC;
        cfg.deposit = PICA_DEPOSIT_DIRECT;
        g.b_ = make(cfg);
        g.dirty_ = true;
    }
    // One context for grid and ensemble with this configuration: reused when it is
    // already theirs; otherwise both host copies are brought up to date under their
    // old contexts and go to a new one.
    template <typename Real, class PA>
    static Binding& bind(YeeGrid<Three, Real>& g, EnsembleSupercells<PA>& e, const pica_config& cfg) {
        if (g.b_ && g.b_ == e.b_ && sameConfig(g.b_->cfg, cfg)) return *g.b_;
        g.read();
        e.ensureHost();
        auto b = make(cfg);
        g.b_ = b;
        g.dirty_ = true;
        e.b_ = b;
        e.dirty_ = true;
        return *b;
    }
    template <typename Real, class PA>
    static void push(YeeGrid<Three, Real>& g, EnsembleSupercells<PA>& e, const pica_config& cfg) {
        Binding& b = bind(g, e, cfg);
        b.settle();
        g.flush();
        e.flush(false);
        check(b.ctx, pica_push_deposit(b.ctx));
        b.pending = true;
        b.fieldsStale = true;
        b.particleEpoch++;
    }
    // A context for the grid alone with this configuration (a flat push): reused when
    // the grid's binding already has it; otherwise the grid's host copy is brought up
    // to date under its old context and goes to a new one.
    template <typename Real>
    static Binding& bindGrid(YeeGrid<Three, Real>& g, const pica_config& cfg) {
        if (g.b_ && sameConfig(g.b_->cfg, cfg)) return *g.b_;
        g.read();
        auto b = make(cfg);
        g.b_ = b;
        g.dirty_ = true;
        return *b;
    }
    template <class PA>
    static void pushFlat(YeeGrid<Three, double>& g, EnsembleUnordered<PA>& e, const pica_config& cfg) {
        Binding& b = bindGrid(g, cfg);
        b.settle();
        g.flush();
        PA& a = e.getParticles();
        const int n = a.size();
        const FP3 lo = e.getMinPosition();
        std::vector<double> v[7];
        for (auto& x : v) x.resize((size_t)n);
        std::vector<int32_t> t((size_t)n);
        for (int i = 0; i < n; i++) {
            const Particle3d q = static_cast<Particle3d>(((const PA&)a)[i]);
            v[0][i] = q.position.x - lo.x; v[1][i] = q.position.y - lo.y; v[2][i] = q.position.z - lo.z;
            v[3][i] = q.p.x; v[4][i] = q.p.y; v[5][i] = q.p.z;
            v[6][i] = q.factor;
            t[(size_t)i] = q.typeIndex;
        }
        check(b.ctx, pica_push_flat_host(b.ctx, n, v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(),
                                         v[5].data(), v[6].data(), t.data(), 0));
        b.fieldsStale = true;
        for (int i = 0; i < n; i++) {
            typename PA::ParticleRef r = a[i];
            r.setPosition(FP3(v[0][i] + lo.x, v[1][i] + lo.y, v[2][i] + lo.z));
            r.setP(FP3(v[3][i], v[4][i], v[5][i]));
        }
    }
    template <typename Real>
    static void fieldUpdate(YeeGrid<Three, Real>& g, double dt, bool electric) {
        if (!g.b_) bindFields(g);
        g.flush();
        check(g.b_->ctx, electric ? pica_update_e(g.b_->ctx, dt) : pica_update_b(g.b_->ctx, dt));
        g.b_->fieldsStale = true;
    }
};
}  // namespace detail

// One step's gather + Boris push + current deposit for every particle of every
// supercell: the supercell loop of a pica host loop, with its per-particle
// fi.get / pusher.push / cd.deposit calls (FieldInterpolatorYeeGrid.h:197-242,
// BorisPusher.h:33-47, CurrentDepositorYeeGrid.h:178-226) replaced by one call.
// The interpolator and the depositor act on one grid; the grid's size equals the
// ensemble's numCells.  J is cleared first.  The migration of the particles that
// left their supercell runs before the next push or read of the ensemble.
template <class PA, class Interpolator, class Particle, typename Real, class Depositor>
void pushSupercells(EnsembleSupercells<PA>& ens, const Interpolator& fi, const BorisPusher<Particle, Real>& pusher,
                    Depositor& cd) {
    static_assert(std::is_same<typename Interpolator::RealType, Real>::value &&
                      std::is_same<typename Depositor::RealType, Real>::value,
                  "the interpolator, the pusher and the depositor take one Real");
    if (static_cast<const void*>(&fi.grid) != static_cast<const void*>(&cd.grid))
        throw Error(PICA_ERR_INVALID, "the interpolator and the depositor act on different grids");
    if (Depositor::shape != 0 && Depositor::shape != Interpolator::shape)
        throw Error(PICA_ERR_INVALID, "the depositor's form factor differs from the interpolator's");
    detail::Access::push(cd.grid, ens,
                         detail::Access::configFor(cd.grid, ens, (double)pusher.dt, Interpolator::shape,
                                                   Depositor::deposit));
}

// One step's gather + Boris push + current deposit for every particle of a flat
// ensemble (EnsembleUnordered, EnsembleOrdered): a pica host loop's per-particle
// fi.get / pusher.push / cd.deposit with the grid-level FieldInterpolatorCIC and
// CurrentDepositorCIC on YeeGrid<Three, double> (FieldInterpolatorYeeGrid.h:137-183,
// BorisPusher.h:33-47, CurrentDepositorYeeGrid.h:126-163), or their TSC siblings,
// replaced by one call (pica_push_flat).  FP64 positions, direct deposition.  The
// grid spans the ensemble's [min, max) (its node 0 at min) and is periodic; each
// particle adds v (q w) / (hx hy hz) to J, which is cleared first; positions wrap
// into [min, max).  The array order does not change.
template <class PA, class Interpolator, class Particle, class Depositor>
void pushParticles(EnsembleUnordered<PA>& ens, const Interpolator& fi, const BorisPusher<Particle, double>& pusher,
                   Depositor& cd) {
    static_assert(std::is_same<typename Interpolator::RealType, double>::value &&
                      std::is_same<typename Depositor::RealType, double>::value,
                  "flat ensembles hold FP64 positions: double operators");
    if (static_cast<const void*>(&fi.grid) != static_cast<const void*>(&cd.grid))
        throw Error(PICA_ERR_INVALID, "the interpolator and the depositor act on different grids");
    if (Depositor::deposit != PICA_DEPOSIT_DIRECT || (Depositor::shape != 0 && Depositor::shape != Interpolator::shape))
        throw Error(PICA_ERR_NOT_BUILT, "flat ensembles deposit directly with the interpolator's form factor");
    auto& g = cd.grid;
    const Int3 n = g.getSize();
    const FP3 h = g.getStep(), span = ens.getMaxPosition() - ens.getMinPosition();
    if (std::fabs(span.x - n.x * h.x) > 1e-9 * span.x || std::fabs(span.y - n.y * h.y) > 1e-9 * span.y ||
        std::fabs(span.z - n.z * h.z) > 1e-9 * span.z)
        throw Error(PICA_ERR_INVALID, "the grid (size times step) must span the ensemble's [min, max)");
    pica_config cfg = detail::Access::base(n, h, (double)pusher.dt, true);
    cfg.sc[0] = cfg.sc[1] = cfg.sc[2] = 1;
    cfg.shape = Interpolator::shape;
    cfg.deposit = PICA_DEPOSIT_DIRECT;
    detail::Access::pushFlat(g, ens, cfg);
}

// pica YeeSolver (fieldSolver/YeeSolver.h:11-38) on the periodic device grid.  A
// grid that no push has bound yet gets a context of its own (fields only).
class YeeSolver {
public:
    template <typename Real>
    void updateE(YeeGrid<Three, Real>& g, double dt) { detail::Access::fieldUpdate(g, dt, true); }
    template <typename Real>
    void updateB(YeeGrid<Three, Real>& g, double dt) { detail::Access::fieldUpdate(g, dt, false); }
};

// ---------------------------------------------------------------------------
// Explicit form: a Simulation built from a Config owns the context; its grid and
// ensemble are bound to it from the start.
// ---------------------------------------------------------------------------
class Simulation {
public:
    typedef YeeGrid<Three, double> Grid;
    typedef EnsembleSupercells<ParticleArraySoA<Particle3d>> Ensemble;

    explicit Simulation(const Config& c)
        : grid_(FP3(0, 0, 0), c.step, c.numCells),
          ens_(FP3(0, 0, 0), FP3(c.numCells.x * c.step.x, c.numCells.y * c.step.y, c.numCells.z * c.step.z),
               c.numCells, c.numCellsPerSupercell) {
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
        b_ = detail::Access::make(cfg);
        // The configured species become pica's global type table (Particle3d::getMass / getCharge).
        ParticleTypes::typesVector = c.types;
        ParticleTypes::types = nullptr;
        ParticleTypes::numTypes = (int)c.types.size();
        dt_ = c.dt;
        detail::Access::attach(grid_, ens_, b_);
    }
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    Grid& grid() { return grid_; }
    Ensemble& ensemble() { return ens_; }
    pica_ctx* handle() { return b_->ctx; }
    double dt() const { return dt_; }
    void setStream(void* cudaStream) { check(b_->ctx, pica_set_stream(b_->ctx, cudaStream)); }
    // One full step: push + deposit, B(dt/2), E(dt), B(dt/2), migrate.
    void step(int n = 1) {
        ready();
        check(b_->ctx, pica_step(b_->ctx, n));
        changed();
    }
    // Push + deposit of every particle (the ensemble then awaits its migration).
    void pushDeposit() {
        ready();
        check(b_->ctx, pica_push_deposit(b_->ctx));
        b_->pending = true;
        changed();
    }
    pica_diag diagnostics(double bgDensity = 0.0) {
        ready();
        pica_diag d{};
        check(b_->ctx, pica_diagnostics(b_->ctx, bgDensity, &d));
        return d;
    }
    int64_t stepCount() { return pica_step_count(b_->ctx); }
    // Synthetic plasma generated on the device in place of ensemble() particles
    // (FP32 cell form; see pica_generate_plasma).
    void generatePlasma(const std::vector<pica_plasma_spec>& specs) {
        b_->settle();
        check(b_->ctx, pica_generate_plasma(b_->ctx, specs.data(), (int32_t)specs.size()));
        detail::Access::replaced(ens_);
        b_->particleEpoch++;
    }
    // Packed particle state of one species (used slots only; see pica_state_packed_slots):
    // statePackedSlots() lays the image out, copyStatePacked() moves one component of
    // it (host: pinned memory of statePackedSlots() x 4 or 8 bytes).
    int64_t statePackedSlots(int species = 0) {
        const int64_t n = pica_state_packed_slots(b_->ctx, species);
        if (n < 0) check(b_->ctx, (int)n);
        return n;
    }
    void copyStatePacked(int species, int comp, void* host, bool toDevice) {
        check(b_->ctx, pica_state_copy_packed(b_->ctx, species, comp, host, toDevice ? 1 : 0));
        if (toDevice) b_->particleEpoch++;
    }
    // The image part of supercells [scBegin, scEnd) (host: start of the whole image);
    // copyStream: the host copy on that cudaStream_t, the gather / scatter kernel on
    // the context stream (pica_state_copy_packed_range_on).
    void copyStatePackedRange(int species, int comp, void* host, bool toDevice, int scBegin, int scEnd,
                              void* copyStream = nullptr) {
        check(b_->ctx, pica_state_copy_packed_range_on(b_->ctx, species, comp, host, toDevice ? 1 : 0, scBegin, scEnd,
                                                       copyStream));
        if (toDevice) b_->particleEpoch++;
    }
    // The push in waitEvents.size() supercell ranges, range r after a wait for
    // waitEvents[r] (cudaEvent_t or nullptr); the rest of the step follows as in a
    // pica host loop: YeeSolver updateB(dt/2), updateE(dt), updateB(dt/2), ensemble().migrate().
    void pushDepositChunked(const std::vector<void*>& waitEvents) {
        check(b_->ctx, pica_push_deposit_chunked(b_->ctx, (int32_t)waitEvents.size(), waitEvents.data()));
        b_->pending = true;
        changed();
    }
    // The same over supercell ranges [bounds[r], bounds[r+1]) of the caller's choice
    // (bounds.size() == waitEvents.size() + 1, from 0 to the supercell count).
    void pushDepositRanges(const std::vector<int32_t>& bounds, const std::vector<void*>& waitEvents) {
        if (bounds.size() != waitEvents.size() + 1) throw Error(PICA_ERR_INVALID, "one more bound than wait events");
        check(b_->ctx, pica_push_deposit_ranges(b_->ctx, (int32_t)waitEvents.size(), bounds.data(), waitEvents.data()));
        b_->pending = true;
        changed();
    }
    // Complete state between steps; a Simulation of the same Config loaded from it
    // continues like this one (FP32 form: bit for bit).
    void saveCheckpoint(const std::string& path) {
        ready();
        check(b_->ctx, pica_checkpoint_save(b_->ctx, path.c_str()));
    }
    void loadCheckpoint(const std::string& path) {
        b_->settle();
        check(b_->ctx, pica_checkpoint_load(b_->ctx, path.c_str()));
        detail::Access::replaced(ens_);
        changed();
    }

private:
    // Host changes to the device, the last migration done.
    void ready() {
        b_->settle();
        detail::Access::flush(grid_);
        detail::Access::flush(ens_);
    }
    void changed() {
        b_->fieldsStale = true;
        b_->particleEpoch++;
    }
    std::shared_ptr<detail::Binding> b_;
    double dt_ = 0;
    Grid grid_;
    Ensemble ens_;
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

// Push + deposit of a Simulation's whole ensemble (pushSupercells with the
// Simulation's own configuration).
inline void pushSupercells(Simulation& sim) { sim.pushDeposit(); }

template <class PA>
std::vector<Particle3d> EnsembleSupercells<PA>::particles() const {
    need();
    const_cast<EnsembleSupercells*>(this)->flush(false);
    return download(nullptr);
}
template <class PA>
std::vector<int32_t> EnsembleSupercells<PA>::counts() const {
    need();
    b_->settle();
    const_cast<EnsembleSupercells*>(this)->flush(false);
    std::vector<int32_t> c((size_t)b_->cfg.nspecies * nsc_.x * nsc_.y * nsc_.z);
    check(b_->ctx, pica_get_counts(b_->ctx, c.data()));
    return c;
}
template <class PA>
std::vector<Particle3d> EnsembleSupercells<PA>::download(std::vector<int32_t>* supercell) const {
    need();
    b_->settle();
    const int64_t n = pica_num_particles(b_->ctx);
    if (n < 0) check(b_->ctx, (int)n);
    std::vector<double> a[7];
    for (auto& v : a) v.resize((size_t)n);
    std::vector<int32_t> t((size_t)n), s((size_t)n);
    check(b_->ctx, pica_download_particles(b_->ctx, a[0].data(), a[1].data(), a[2].data(), a[3].data(), a[4].data(),
                                           a[5].data(), a[6].data(), t.data(), s.data()));
    std::vector<Particle3d> out((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        out[i].position = FP3(a[0][i], a[1][i], a[2][i]) + min_;
        out[i].p = FP3(a[3][i], a[4][i], a[5][i]);
        out[i].factor = a[6][i];
        out[i].typeIndex = (short)t[i];
    }
    if (supercell) *supercell = std::move(s);
    return out;
}

}  // namespace pica_gb300
