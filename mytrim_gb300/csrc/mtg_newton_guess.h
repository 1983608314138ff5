// Geometry of the FP32 path's first-guess table for the distance of closest
// approach (host and device).  For each screened potential the table holds
// log2(r0 - b), r0 the converged root of b^2 / r + phi(r) / eps - r = 0
// (trim.C:192-233), on a grid uniform in log2(eps) and in b.  The FP32 Newton
// solve starts from the bilinear interpolation of this table inside the grid and
// from the reference's guess (trim.C:183-190) outside it; its steps and its
// stopping test are unchanged.  The C-Kr potential keeps the reference's guess
// everywhere: its derivative coefficients as the reference writes them are not
// the derivative's, so the iteration converges slowly and where it stops depends
// on where it starts.
#pragma once

namespace mtg
{

constexpr int NG_U = 64;               // log2(eps) rows
constexpr int NG_B = 64;               // b columns
constexpr int NG_POT = 2;              // universal, Moliere
constexpr double NG_U0 = -18.0;        // log2(eps) of the first row
constexpr double NG_U1 = 3.32192809488736235; // log2(10): above eps = 10 the asymptotic branch applies
constexpr double NG_BMAX = 32.0;       // b of the last column
constexpr double NG_DU = (NG_U1 - NG_U0) / (NG_U - 1);
constexpr double NG_DB = NG_BMAX / (NG_B - 1);
constexpr int NG_CELLS = NG_POT * NG_U * NG_B;

} // namespace mtg
