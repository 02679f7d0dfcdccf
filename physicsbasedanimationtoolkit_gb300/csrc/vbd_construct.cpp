// Host precompute of a VBD problem: the work of sim::vbd::Data::Construct
// (sim/vbd/Data.cpp:179-243 of the reference), done once per mesh in FP64 before the upload.
//
//   * lumped mass  m_i = sum_{e ni i} rho_e V_e / 4      (fem/Mass.h:357-397, Data.cpp:210-219)
//   * shape-function gradients of the linear tet        (fem/ShapeFunctions.h:267-296)
//   * quadrature weight wg_e = V_e                      (fem/MeshQuadrature.h:75-88)
//   * vertex -> tet adjacency, tets ascending           (Data.cpp:223-226)
//   * greedy colouring of the vertex graph              (graph/Color.h:45-135), bit-exact with the
//     reference: visiting order = stable sort by degree (incl. the vertex itself), colour = the
//     least used (or first) usable colour, ties to the lowest colour index
//   * colour partitions minus Dirichlet vertices        (graph/Adjacency.h:172-181, 307-342)
#include "vbd_construct.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace pbgb {

namespace {

double det_cols(double const* a, double const* b, double const* c)
{
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - b[0] * (a[1] * c[2] - a[2] * c[1]) +
           c[0] * (a[1] * b[2] - a[2] * b[1]);
}

} // namespace

int construct(ConstructIn const& in, ConstructOut& out)
{
    int32_t const nV = in.nV, nT = in.nT;
    if (nV < 0 || nT < 0 || (nV > 0 && !in.X) || (nT > 0 && (!in.T || !in.rhoe)))
        return kInvalid;
    for (int64_t k = 0; k < int64_t(nT) * 4; ++k)
        if (in.T[k] < 0 || in.T[k] >= nV)
            return kInvalid;
    if (in.ordering < 0 || in.ordering > 2 || in.selection < 0 || in.selection > 1)
        return kInvalid;

    // --- element geometry and lumped mass ------------------------------------------------------
    std::fill(out.m, out.m + nV, 0.0);
    for (int32_t e = 0; e < nT; ++e)
    {
        int32_t const* t = in.T + 4 * size_t(e);
        double const* X0 = in.X + 3 * size_t(t[0]);
        double a[3], b[3], c[3];
        for (int r = 0; r < 3; ++r)
        {
            a[r] = in.X[3 * size_t(t[1]) + r] - X0[r];
            b[r] = in.X[3 * size_t(t[2]) + r] - X0[r];
            c[r] = in.X[3 * size_t(t[3]) + r] - X0[r];
        }
        double const detJ = det_cols(a, b, c);
        if (!(detJ > 0.0))
            return kDegenerate;
        // J^-1 rows are (b x c, c x a, a x b) / det; GP row q (q = 1..3) is row q-1 of J^-1.
        double r1[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
        double r2[3] = {c[1] * a[2] - c[2] * a[1], c[2] * a[0] - c[0] * a[2], c[0] * a[1] - c[1] * a[0]};
        double r3[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double* G     = out.GP + 12 * size_t(e);
        double const s = 1.0 / detJ;
        for (int d = 0; d < 3; ++d)
        {
            G[3 + d] = r1[d] * s;
            G[6 + d] = r2[d] * s;
            G[9 + d] = r3[d] * s;
            G[d]     = -(G[3 + d] + G[6 + d] + G[9 + d]);
        }
        double const vol = detJ / 6.0;
        out.wg[e]        = vol;
        double const me  = in.rhoe[e] * vol * 0.25;
        for (int q = 0; q < 4; ++q)
            out.m[t[q]] += me;
    }

    // --- vertex -> tet adjacency ------------------------------------------------------------------
    std::fill(out.GVGp, out.GVGp + nV + 1, 0);
    for (int64_t k = 0; k < int64_t(nT) * 4; ++k)
        out.GVGp[in.T[k] + 1]++;
    std::partial_sum(out.GVGp, out.GVGp + nV + 1, out.GVGp);
    {
        std::vector<int32_t> cursor(out.GVGp, out.GVGp + nV);
        for (int32_t e = 0; e < nT; ++e)
            for (int q = 0; q < 4; ++q)
            {
                int32_t const v = in.T[4 * size_t(e) + q];
                int32_t const k = cursor[v]++;
                out.GVGe[k]      = e;
                out.GVGilocal[k] = q;
            }
    }

    // --- vertex graph degrees (distinct neighbours incl. self) and neighbour lists -------------
    std::vector<int32_t> nbrPtr(size_t(nV) + 1, 0);
    std::vector<int32_t> nbr;
    nbr.reserve(size_t(out.GVGp[nV]) * 2);
    {
        std::vector<int32_t> stamp(size_t(nV), -1);
        for (int32_t v = 0; v < nV; ++v)
        {
            for (int32_t k = out.GVGp[v]; k < out.GVGp[v + 1]; ++k)
            {
                int32_t const* t = in.T + 4 * size_t(out.GVGe[k]);
                for (int q = 0; q < 4; ++q)
                    if (stamp[t[q]] != v)
                    {
                        stamp[t[q]] = v;
                        nbr.push_back(t[q]);
                    }
            }
            nbrPtr[v + 1] = int32_t(nbr.size());
        }
    }

    // --- greedy colouring --------------------------------------------------------------------------
    std::vector<int32_t> visit(static_cast<size_t>(nV));
    std::iota(visit.begin(), visit.end(), 0);
    if (in.ordering != 0)
    {
        bool const largest = in.ordering == 2;
        std::stable_sort(visit.begin(), visit.end(), [&](int32_t a, int32_t b) {
            int32_t const da = nbrPtr[a + 1] - nbrPtr[a];
            int32_t const db = nbrPtr[b + 1] - nbrPtr[b];
            return largest ? da > db : da < db;
        });
    }
    std::fill(out.colors, out.colors + nV, -1);
    std::vector<int32_t> used;     // vertices per colour
    std::vector<int32_t> blocked;  // colour -> last vertex that blocked it
    for (int32_t u : visit)
    {
        int nBlocked = 0;
        for (int32_t k = nbrPtr[u]; k < nbrPtr[u + 1]; ++k)
        {
            int32_t const c = out.colors[nbr[k]];
            if (c >= 0 && blocked[c] != u)
            {
                blocked[c] = u;
                ++nBlocked;
            }
        }
        int32_t const nC = int32_t(used.size());
        if (nBlocked == nC)
        {
            if (nC == kMaxColors)
                return kPalette;
            out.colors[u] = nC;
            used.push_back(1);
            blocked.push_back(-1);
            continue;
        }
        int32_t best = -1;
        for (int32_t c = 0; c < nC; ++c)
        {
            if (blocked[c] == u)
                continue;
            if (best < 0 || (in.selection == 0 && used[c] < used[best]))
                best = c;
            if (in.selection == 1)
                break;
        }
        out.colors[u] = best;
        ++used[best];
    }

    // --- partitions without Dirichlet vertices ----------------------------------------------------
    std::vector<char> pinned(size_t(nV), 0);
    for (int32_t k = 0; k < in.nDbc; ++k)
    {
        if (in.dbc[k] < 0 || in.dbc[k] >= nV)
            return kInvalid;
        pinned[in.dbc[k]] = 1;
    }
    int32_t const nC = int32_t(used.size());
    std::vector<int32_t> cursor(size_t(nC) + 1, 0);
    for (int32_t v = 0; v < nV; ++v)
        if (!pinned[v])
            cursor[out.colors[v] + 1]++;
    std::partial_sum(cursor.begin(), cursor.end(), cursor.begin());
    for (int32_t c = 0; c <= nC; ++c)
        out.Pptr[c] = cursor[c];
    for (int32_t v = 0; v < nV; ++v)
        if (!pinned[v])
            out.Padj[cursor[out.colors[v]]++] = v;
    out.nPartitions = nC;
    out.nPadj       = out.Pptr[nC];
    return kOk;
}

} // namespace pbgb
