// Drives the C++ facade (include/pbat_gb300.hpp) the way code written against the reference's
// pbat::gpu::vbd::Integrator does, from an object with the reference Data's member names.
//
//   facade_main <mesh.txt> <out.txt> <steps> <iterations>
// mesh.txt: "nV nT nDbc", then nV lines "x y z", nT lines "a b c d", nDbc vertex indices.
// Writes the positions after the steps (3 x nV, one vertex per line, %.9g).  Exit codes: 0 ok,
// 3 no CUDA device (the error is printed), 2 bad arguments, 1 other failures.
#define PBGB_PROVIDE_PBAT_NAMESPACE
#include "pbat_gb300.hpp"

#include <cstdio>
#include <fstream>
#include <vector>

namespace {

// Minimal column-major matrix with the members the facade reads.
template <class T>
struct Mat
{
    std::int64_t r = 0, c = 0;
    std::vector<T> v;
    Mat() = default;
    Mat(std::int64_t rows, std::int64_t cols) : r(rows), c(cols), v(std::size_t(rows * cols)) {}
    T* data() { return v.data(); }
    T const* data() const { return v.data(); }
    std::int64_t size() const { return r * c; }
    std::int64_t cols() const { return c; }
    T& operator()(std::int64_t i, std::int64_t j) { return v[std::size_t(j * r + i)]; }
};

enum class EInitializationStrategy { Position, Inertia, KineticEnergyMinimum, AdaptiveVbd, AdaptivePbat };
enum class EAccelerationStrategy { None, Chebyshev };

// The reference Data's member names (sim/vbd/Data.h:164-245); Index = std::ptrdiff_t there.
struct Data
{
    Mat<double> X, x, v, aext, lame;
    Mat<std::ptrdiff_t> E, V, F, B, Pptr, Padj;
    Mat<double> m, wg, XVA, FA;
    EInitializationStrategy strategy{EInitializationStrategy::KineticEnergyMinimum};
    double kD{0}, detHZero{1e-7}, rho{1}, muC{1e6}, muF{0.3}, epsv{1e-3};
    std::ptrdiff_t mActiveSetUpdateFrequency{1};
    std::ptrdiff_t mWindowSize{5};
    double mNesterovLipschitzConstant{1};
    std::ptrdiff_t mNesterovAccelerationStart{3};
    double eta{0.2}, tau{2};
    bool bCurved{true};
    EAccelerationStrategy eAcceleration{EAccelerationStrategy::None};
};

} // namespace

int main(int argc, char** argv)
{
    if (argc != 5)
        return 2;
    std::ifstream in(argv[1]);
    std::int64_t nV = 0, nT = 0, nD = 0;
    in >> nV >> nT >> nD;
    Data d;
    d.X = Mat<double>(3, nV);
    for (std::int64_t i = 0; i < nV; ++i)
        in >> d.X(0, i) >> d.X(1, i) >> d.X(2, i);
    d.E = Mat<std::ptrdiff_t>(4, nT);
    std::vector<std::int32_t> T(std::size_t(4 * nT));
    for (std::int64_t e = 0; e < nT; ++e)
        for (int k = 0; k < 4; ++k)
        {
            in >> d.E(k, e);
            T[std::size_t(4 * e + k)] = std::int32_t(d.E(k, e));
        }
    std::vector<std::int32_t> dbc(static_cast<std::size_t>(nD));
    for (auto& q : dbc)
        in >> q;
    if (!in)
        return 2;
    // Data::Construct through the C ABI (masses, GP, wg, colouring, partitions).
    std::size_t const sV = static_cast<std::size_t>(nV), sT = static_cast<std::size_t>(nT);
    std::vector<double> rho(sT, 1000.0), m(sV), GP(12 * sT), wg(sT);
    std::vector<std::int32_t> GVGp(sV + 1), GVGe(4 * sT), GVGl(4 * sT), colors(sV), Pptr(129), Padj(sV);
    std::int32_t nP = 0, nPadj = 0;
    int rc = pbgb_vbd_data_construct(std::int32_t(nV), std::int32_t(nT), d.X.data(), T.data(), rho.data(), dbc.data(),
                                     std::int32_t(nD), 2, 0, m.data(), GP.data(), wg.data(), GVGp.data(), GVGe.data(),
                                     GVGl.data(), colors.data(), Pptr.data(), &nP, Padj.data(), &nPadj);
    if (rc != PBGB_OK)
    {
        std::fprintf(stderr, "construct failed: %s\n", pbgb_last_error(nullptr));
        return 1;
    }
    d.x    = d.X;
    d.v    = Mat<double>(3, nV);
    d.aext = Mat<double>(3, nV);
    for (std::int64_t i = 0; i < nV; ++i)
        d.aext(2, i) = -9.81;
    for (auto q : dbc)
        d.aext(2, q) = 0.0;
    d.m  = Mat<double>(nV, 1);
    d.m.v = m;
    d.wg  = Mat<double>(nT, 1);
    d.wg.v = wg;
    d.lame = Mat<double>(2, nT);
    double const E = 1e6, nu = 0.45;
    for (std::int64_t e = 0; e < nT; ++e)
    {
        d.lame(0, e) = E / (2 * (1 + nu));
        d.lame(1, e) = E * nu / ((1 + nu) * (1 - 2 * nu));
    }
    d.Pptr = Mat<std::ptrdiff_t>(nP + 1, 1);
    for (std::int32_t k = 0; k <= nP; ++k)
        d.Pptr.v[std::size_t(k)] = Pptr[std::size_t(k)];
    d.Padj = Mat<std::ptrdiff_t>(nPadj, 1);
    for (std::int32_t k = 0; k < nPadj; ++k)
        d.Padj.v[std::size_t(k)] = Padj[std::size_t(k)];
    try
    {
        pbat::gpu::vbd::Integrator vbd(d);
        vbd.SetBlockSize(64);
        vbd.SetInitializationStrategy(EInitializationStrategy::KineticEnergyMinimum);
        int const steps = std::atoi(argv[3]), iterations = std::atoi(argv[4]);
        for (int s = 0; s < steps; ++s)
            vbd.Step(1.f / 60.f, iterations, 1);
        auto x = vbd.GetPositions();
        std::FILE* out = std::fopen(argv[2], "w");
        if (!out)
            return 1;
        for (std::int64_t i = 0; i < nV; ++i)
            std::fprintf(out, "%.9g %.9g %.9g\n", x(0, i), x(1, i), x(2, i));
        std::fclose(out);
    }
    catch (pbgb::Error const& e)
    {
        std::fprintf(stderr, "pbgb error %d: %s\n", e.code(), e.what());
        return e.code() == PBGB_ERR_NO_DEVICE ? 3 : 1;
    }
    return 0;
}
