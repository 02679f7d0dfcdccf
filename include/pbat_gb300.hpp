/*
 * C++ facade over the C ABI of pbat_gb300.h with the reference's public GPU integrator interface:
 * pbat::gpu::vbd::Integrator (gpu/vbd/Integrator.h:33-148) -- Step, SetPositions, SetVelocities,
 * SetExternalAcceleration, SetNumericalZeroForHessianDeterminant, SetRayleighDampingCoefficient,
 * SetInitializationStrategy, SetBlockSize, SetSceneBoundingBox, GetPositions, GetVelocities --
 * move-only, throwing on failure like the reference.
 *
 * Header-only, C++17, no Eigen dependency:
 *   - the constructor takes the reference's own pbat::sim::vbd::Data after Construct() (or any
 *     object with the same member names: x, X, E, v, aext, m, wg, lame, Pptr, Padj, strategy, kD,
 *     detHZero, eAcceleration, rho, mWindowSize, mNesterovLipschitzConstant,
 *     mNesterovAccelerationStart, eta, tau, bCurved, and for contact V, F, B, XVA, FA, muC, muF, epsv,
 *     mActiveSetUpdateFrequency), reading each member through data()/size()/cols();
 *   - matrices passed in are any column-major 3 x n float matrix with data() and cols() (Eigen's
 *     GpuMatrixX, Eigen::Ref<GpuMatrixX const>, or pbgb::Matrix3X);
 *   - GetPositions<M>() / GetVelocities<M>() return an M constructed as M(3, n) with data();
 *     the default M is pbgb::Matrix3X (GetPositions<GpuMatrixX>() gives the reference's type).
 *
 * Defining PBGB_PROVIDE_PBAT_NAMESPACE before including this header also declares
 * pbat::gpu::vbd::Integrator as this class, for code that names the reference's type directly.
 */
#pragma once

#include "pbat_gb300.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace pbgb {

// A failing C ABI call: the status code and pbgb_last_error's message.
class Error : public std::runtime_error
{
  public:
    Error(int code, std::string const& what) : std::runtime_error(what), code_(code) {}
    int code() const noexcept { return code_; }

  private:
    int code_;
};

inline void Check(int rc, pbgb_vbd* h)
{
    if (rc != PBGB_OK)
    {
        char const* msg = pbgb_last_error(h);
        throw Error(rc, msg ? msg : "pbgb: unknown error");
    }
}

// Column-major 3 x n float matrix (used when no Eigen type is requested).
struct Matrix3X
{
    Matrix3X() = default;
    Matrix3X(std::int64_t rows, std::int64_t cols) : n(cols), values(std::size_t(rows * cols), 0.f)
    {
        if (rows != 3)
            throw std::invalid_argument("pbgb::Matrix3X has 3 rows");
    }
    float* data() { return values.data(); }
    float const* data() const { return values.data(); }
    std::int64_t rows() const { return 3; }
    std::int64_t cols() const { return n; }
    std::int64_t size() const { return 3 * n; }
    float& operator()(std::int64_t r, std::int64_t c) { return values[std::size_t(3 * c + r)]; }
    float operator()(std::int64_t r, std::int64_t c) const { return values[std::size_t(3 * c + r)]; }

    std::int64_t n = 0;
    std::vector<float> values;
};

namespace detail {

template <class TVector>
std::vector<std::int32_t> to_int32(TVector const& v)
{
    std::vector<std::int32_t> out(static_cast<std::size_t>(v.size()));
    for (std::size_t k = 0; k < out.size(); ++k)
        out[k] = static_cast<std::int32_t>(v.data()[k]);
    return out;
}

template <class TVector>
std::vector<double> to_double(TVector const& v)
{
    std::vector<double> out(static_cast<std::size_t>(v.size()));
    for (std::size_t k = 0; k < out.size(); ++k)
        out[k] = static_cast<double>(v.data()[k]);
    return out;
}

} // namespace detail

namespace vbd {

class Integrator
{
  public:
    // From a constructed reference Data (sim/vbd/Data.h:164-245): positions, elements, masses,
    // quadrature weights, Lame coefficients, partitions and solver settings.
    template <class TData>
    explicit Integrator(TData const& data)
    {
        std::int32_t const nV = static_cast<std::int32_t>(data.x.cols());
        std::int32_t const nT = static_cast<std::int32_t>(data.E.cols());
        std::vector<double> x = detail::to_double(data.x), X = detail::to_double(data.X);
        std::vector<double> v = detail::to_double(data.v), a = detail::to_double(data.aext);
        std::vector<double> m = detail::to_double(data.m), wg = detail::to_double(data.wg);
        std::vector<double> lame = detail::to_double(data.lame); // 2 x nT column-major
        std::vector<double> mu(static_cast<std::size_t>(nT)), lambda(static_cast<std::size_t>(nT));
        for (std::int32_t e = 0; e < nT; ++e)
        {
            mu[e]     = lame[2 * std::size_t(e)];
            lambda[e] = lame[2 * std::size_t(e) + 1];
        }
        std::vector<std::int32_t> T = detail::to_int32(data.E), Pptr = detail::to_int32(data.Pptr);
        std::vector<std::int32_t> Padj = detail::to_int32(data.Padj);
        pbgb_vbd_desc d{};
        d.n_vertices        = nV;
        d.n_tets            = nT;
        d.x                 = x.data();
        d.X                 = X.data();
        d.T                 = T.data();
        d.v                 = v.data();
        d.aext              = a.data();
        d.m                 = m.data();
        d.wg                = wg.data();
        d.mu                = mu.data();
        d.lambda            = lambda.data();
        d.n_partitions      = static_cast<std::int32_t>(Pptr.size()) - 1;
        d.Pptr              = Pptr.data();
        d.Padj              = Padj.data();
        d.init_strategy     = static_cast<std::int32_t>(data.strategy);
        d.kD                = static_cast<double>(data.kD);
        d.detHZero          = static_cast<double>(data.detHZero);
        // gpu/vbd/Integrator.cu:15-33 builds Anderson, Chebyshev and trust-region integrators and
        // the base integrator for every other strategy (Nesterov and Broyden included).
        std::int32_t const accel = static_cast<std::int32_t>(data.eAcceleration);
        d.acceleration = (accel == PBGB_ACCEL_CHEBYSHEV || accel == PBGB_ACCEL_ANDERSON ||
                          accel == PBGB_ACCEL_TRUST_REGION) ? accel : PBGB_ACCEL_NONE;
        d.rho               = static_cast<double>(data.rho);
        d.window_size       = static_cast<std::int32_t>(data.mWindowSize);
        d.nesterov_lipschitz = static_cast<double>(data.mNesterovLipschitzConstant);
        d.nesterov_start     = static_cast<std::int32_t>(data.mNesterovAccelerationStart);
        d.tr_eta             = static_cast<double>(data.eta);
        d.tr_tau             = static_cast<double>(data.tau);
        d.tr_curved          = data.bCurved ? 1 : 0;
        d.chebyshev_formula = PBGB_CHEBYSHEV_REFERENCE;
        d.semantics         = PBGB_SEMANTICS_GPU;
        std::vector<std::int32_t> V, F, B;
        std::vector<double> XVA, FA;
        if (data.F.size() > 0)
        {
            V   = detail::to_int32(data.V);
            F   = detail::to_int32(data.F); // 3 x nF column-major: triangle-major
            B   = detail::to_int32(data.B);
            XVA = detail::to_double(data.XVA);
            FA  = detail::to_double(data.FA);
            d.n_collision_vertices        = static_cast<std::int32_t>(V.size());
            d.V                           = V.data();
            d.n_collision_triangles       = static_cast<std::int32_t>(F.size() / 3);
            d.F                           = F.data();
            d.B                           = B.data();
            d.XVA                         = XVA.data();
            d.FA                          = FA.data();
            d.muC                         = static_cast<double>(data.muC);
            d.muF                         = static_cast<double>(data.muF);
            d.epsv                        = static_cast<double>(data.epsv);
            d.active_set_update_frequency = static_cast<std::int32_t>(data.mActiveSetUpdateFrequency);
        }
        Check(pbgb_vbd_create(&d, &h_), nullptr);
        nV_ = nV;
    }

    // From a filled descriptor (one mesh) or several (the batched form).
    explicit Integrator(pbgb_vbd_desc const& desc) : nV_(desc.n_vertices)
    {
        Check(pbgb_vbd_create(&desc, &h_), nullptr);
    }
    Integrator(pbgb_vbd_desc const* descs, std::int32_t n_meshes)
    {
        Check(pbgb_vbd_create_batched(descs, n_meshes, &h_), nullptr);
        std::int32_t nT = 0, nF = 0, nC = 0;
        Check(pbgb_vbd_sizes(h_, &nV_, &nT, &nF, &nC), h_);
    }

    Integrator(Integrator const&)            = delete;
    Integrator& operator=(Integrator const&) = delete;
    Integrator(Integrator&& o) noexcept : h_(std::exchange(o.h_, nullptr)), nV_(o.nV_) {}
    Integrator& operator=(Integrator&& o) noexcept
    {
        if (this != &o)
        {
            pbgb_vbd_destroy(h_);
            h_  = std::exchange(o.h_, nullptr);
            nV_ = o.nV_;
        }
        return *this;
    }
    ~Integrator() { pbgb_vbd_destroy(h_); }

    void Step(float dt, std::int32_t iterations, std::int32_t substeps = 1)
    {
        Check(pbgb_vbd_step(h_, dt, iterations, substeps), h_);
    }

    template <class TMatrix>
    void SetPositions(TMatrix const& X)
    {
        Check(pbgb_vbd_set_positions(h_, checked(X)), h_);
        Check(pbgb_vbd_synchronize(h_), h_);
    }
    template <class TMatrix>
    void SetVelocities(TMatrix const& v)
    {
        Check(pbgb_vbd_set_velocities(h_, checked(v)), h_);
        Check(pbgb_vbd_synchronize(h_), h_);
    }
    template <class TMatrix>
    void SetExternalAcceleration(TMatrix const& aext)
    {
        Check(pbgb_vbd_set_external_acceleration(h_, checked(aext)), h_);
        Check(pbgb_vbd_synchronize(h_), h_);
    }
    void SetNumericalZeroForHessianDeterminant(float zero) { Check(pbgb_vbd_set_detH_zero(h_, zero), h_); }
    void SetRayleighDampingCoefficient(float kD) { Check(pbgb_vbd_set_damping(h_, kD), h_); }
    template <class TStrategy>
    void SetInitializationStrategy(TStrategy strategy)
    {
        Check(pbgb_vbd_set_strategy(h_, static_cast<std::int32_t>(strategy)), h_);
    }
    void SetBlockSize(std::int32_t blockSize) { Check(pbgb_vbd_set_block_size(h_, blockSize), h_); }
    template <class TVector>
    void SetSceneBoundingBox(TVector const& min, TVector const& max)
    {
        float const lo[3] = {float(min.data()[0]), float(min.data()[1]), float(min.data()[2])};
        float const hi[3] = {float(max.data()[0]), float(max.data()[1]), float(max.data()[2])};
        Check(pbgb_vbd_set_scene_bounding_box(h_, lo, hi), h_);
    }

    template <class TMatrix = Matrix3X>
    TMatrix GetPositions() const
    {
        TMatrix x(3, nV_);
        Check(pbgb_vbd_get_positions(h_, x.data()), h_);
        return x;
    }
    template <class TMatrix = Matrix3X>
    TMatrix GetVelocities() const
    {
        TMatrix v(3, nV_);
        Check(pbgb_vbd_get_velocities(h_, v.data()), h_);
        return v;
    }

    // The underlying C handle (for the calls beyond the reference's interface).
    pbgb_vbd* handle() const { return h_; }
    std::int32_t NumVertices() const { return nV_; }

  private:
    template <class TMatrix>
    float const* checked(TMatrix const& M) const
    {
        if (static_cast<std::int64_t>(M.cols()) != nV_ || static_cast<std::int64_t>(M.size()) != 3 * std::int64_t(nV_))
            throw std::invalid_argument("expected a 3 x |#vertices| column-major float matrix");
        return M.data();
    }

    pbgb_vbd* h_     = nullptr;
    std::int32_t nV_ = 0;
};

} // namespace vbd
} // namespace pbgb

#ifdef PBGB_PROVIDE_PBAT_NAMESPACE
namespace pbat::gpu::vbd {
using Integrator = ::pbgb::vbd::Integrator;
} // namespace pbat::gpu::vbd
#endif
