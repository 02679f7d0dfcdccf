// Host precompute of a VBD problem (sim::vbd::Data::Construct of the reference).
#pragma once
#include <cstdint>

namespace pbgb {

enum Status : int
{
    kOk        = 0,
    kInvalid   = 1,
    kCuda      = 2,
    kNonFinite = 3,
    kDegenerate = 4,
    kPalette   = 5,
    kNoDevice  = 6,
    kTimeout   = 7,
    kInternal  = 8,
};

int constexpr kMaxColors = 128;

struct ConstructIn
{
    int32_t nV;
    int32_t nT;
    double const* X;  // nV x 3
    int32_t const* T; // nT x 4
    double const* rhoe;
    int32_t const* dbc;
    int32_t nDbc;
    int32_t ordering;  // 0 natural, 1 smallest degree, 2 largest degree
    int32_t selection; // 0 least used, 1 first available
};

struct ConstructOut
{
    double* m;
    double* GP; // nT x 4 x 3, row a = grad N_a
    double* wg;
    int32_t* GVGp;
    int32_t* GVGe;
    int32_t* GVGilocal;
    int32_t* colors;
    int32_t* Pptr; // >= kMaxColors + 1
    int32_t* Padj; // >= nV
    int32_t nPartitions;
    int32_t nPadj;
};

int construct(ConstructIn const& in, ConstructOut& out);

} // namespace pbgb
