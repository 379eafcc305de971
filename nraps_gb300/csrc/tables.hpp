/* tables.hpp — byte offsets of the packed device tables of one problem. */
#ifndef NRAPS_TABLES_HPP
#define NRAPS_TABLES_HPP
#include <cstddef>
#include <string>
#include <vector>
#include <cstdint>

#include "../../include/nraps_gpu.h"

struct TableLayout {
    size_t sigt, sigs, siga, inv_sigtr, nsf, nsf_sigtr, pabs, scat, chi_cdf, phys_cdf;
    size_t left, right, dx, mat, fuel, nsf64, dx64;
    size_t total;
    double conv_const;
};

/* Tables of the event-based Woodcock engine for one problem instance (FP32).
   Material regions are maximal runs of cells with the same matid and the same
   (bitwise) width, so a cell index inside a region is arithmetic.
     sigtr  = f32(sigt - mu*sigs) evaluated in FP64 (exact product)
     pabs   = siga / sigtr,  nsf_st = (nut*sigf) / sigtr,  inv_st = 1 / sigtr
     ocdf   = outcome CDF of a real collision, G entries per (m, g): entry 0 is
              pabs (absorbed), entry e >= 1 is pabs + (1 - pabs) * scdf[e-1]
              (scattered into a group below e), scdf being the
              transport-corrected scatter CDF (within-group term minus
              mu*sigs); one uniform u picks the outcome: absorbed if
              u < ocdf[0], else group (number of entries <= u) - 1
     maj[g] = max of sigtr over the materials present, maj[G+g] = 1/maj[g]
     rdat   = per region (R+1 entries, the last holds left = L): left edge,
              1/cell width, first cell, cells (the last two as u32 bits)
     bins   = nbins equal bins of [0, L]; bin b holds the first region r0 any
              x with (int)(x * inv_binw) == b can lie in, the next region's
              left edge x1 (r = r0 + (x >= x1)), and bit 31 of the region
              word set when the bin holds more than one region boundary
              (then the lookup walks on)                                    */
struct EvHostTables {
    uint32_t M = 0, G = 0, R = 0, nc = 0, nbins = 0, nfuel = 0;
    float L = 0.f, inv_binw = 0.f, boundl = 0.f, boundr = 0.f;
    std::vector<float> xs, scdf, ocdf, chicdf, maj, rleft, rinvdx, cleft, cdx;
    std::vector<float> rdat;            /* 4 per region, R+1 regions            */
    std::vector<uint8_t> rmat, cmat;
    std::vector<uint32_t> rfirst, rncell, fuel;
    std::vector<uint32_t> bins;         /* 2 per bin: x1 bits, r0 | multi << 31 */
    std::vector<double> nsf64, dx64, inv_dx64;
    std::vector<double> inv_st64;       /* [m*G+g] (double)(1/sigtr): flux score  */
    std::vector<uint64_t> kq;           /* [m*G+g] nsf_st in 2^-32 fixed point    */
    double conv_const = 0.0;
};
int build_event_tables(const nraps_problem& p, EvHostTables& t, std::string& err);

/* Returns 0 on success, else fills err. */
template <class T>
int build_tables(const nraps_problem& p, std::vector<unsigned char>& blob, TableLayout& L,
                 std::string& err);
#endif
