/* tables.hpp — byte offsets of the packed device tables of one problem. */
#ifndef NRAPS_TABLES_HPP
#define NRAPS_TABLES_HPP
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/nraps_gpu.h"

struct TableLayout {
    size_t sigt, sigs, siga, inv_sigtr, nsf, nsf_sigtr, pabs, scat, chi_cdf, phys_cdf;
    size_t left, right, dx, mat, fuel, nsf64, dx64;
    size_t total;
    double conv_const;
};

/* Returns 0 on success, else fills err. */
template <class T>
int build_tables(const nraps_problem& p, std::vector<unsigned char>& blob, TableLayout& L,
                 std::string& err);
#endif
