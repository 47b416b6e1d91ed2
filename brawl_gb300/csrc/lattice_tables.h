// lattice_tables.h -- coordination-shell neighbour vectors of the three
// BraWl lattices, in the exact order the reference adds them.
//
// Each entry is a (dx, dy, dz) step on the doubled cubic grid that BraWl uses
// to represent every lattice (config(1, 2n1, 2n2, 2n3)).  The order inside a
// shell is the order of the nbrs(:) assignments in the reference's
// {bcc,fcc,simple_cubic}_shellN_energy functions, and the order matters: the
// reference adds V_ex one neighbour at a time, so this order fixes how every
// FP64 site energy rounds.
//   bcc shells 1-10 : src/bw_hamiltonian.f90:134-877
//   fcc shells 1-6  : src/bw_hamiltonian.f90:1282-1691
//   sc  shells 1-2  : src/bw_hamiltonian.f90:1930-2038
// Two reference quirks are kept on purpose: bcc shell 8 contains two entries,
// (0,4,0) and (-4,0,0), that lie on shell 6, and bcc shell 10 repeats four of
// its entries.  The simple-cubic routines wrap neighbour indices modulo n
// rather than 2n; the wrapping rule lives with the kernels, not here.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define BRAWL_TABLE static constexpr
#else
#define BRAWL_TABLE static constexpr
#endif

namespace brawl {

enum Lattice : int { kSimpleCubic = 0, kBcc = 1, kFcc = 2 };

// sc: 2 shells, 18 entries
BRAWL_TABLE int8_t kSCOffsets[18][3] = {
    {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},  // shell 1
    {0, 1, -1}, {-1, 0, -1}, {1, 0, -1}, {0, -1, -1}, {1, 1, 0}, {-1, 1, 0},
    {1, -1, 0}, {-1, -1, 0}, {0, 1, 1}, {-1, 0, 1}, {1, 0, 1}, {0, -1, 1},  // shell 2
};
BRAWL_TABLE int16_t kSCShellStart[3] = {0, 6, 18};

// bcc: 10 shells, 168 entries
BRAWL_TABLE int8_t kBCCOffsets[168][3] = {
    {1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1},
    {-1, -1, -1},  // shell 1
    {2, 0, 0}, {-2, 0, 0}, {0, -2, 0}, {0, 2, 0}, {0, 0, 2}, {0, 0, -2},  // shell 2
    {0, -2, -2}, {2, 0, -2}, {-2, 0, -2}, {0, 2, -2}, {2, -2, 0}, {-2, -2, 0}, {2, 2, 0},
    {-2, 2, 0}, {0, -2, 2}, {2, 0, 2}, {-2, 0, 2}, {0, 2, 2},  // shell 3
    {1, 1, 3}, {-1, 1, 3}, {1, -1, 3}, {-1, -1, 3}, {1, 1, -3}, {-1, 1, -3}, {1, -1, -3},
    {-1, -1, -3}, {1, 3, 1}, {-1, 3, 1}, {1, 3, -1}, {-1, 3, -1}, {1, -3, 1}, {-1, -3, 1},
    {1, -3, -1}, {-1, -3, -1}, {3, 1, 1}, {3, -1, 1}, {3, 1, -1}, {3, -1, -1}, {-3, 1, 1},
    {-3, -1, 1}, {-3, 1, -1}, {-3, -1, -1},  // shell 4
    {2, 2, 2}, {-2, 2, 2}, {2, -2, 2}, {-2, -2, 2}, {2, 2, -2}, {-2, 2, -2}, {2, -2, -2},
    {-2, -2, -2},  // shell 5
    {4, 0, 0}, {-4, 0, 0}, {0, 4, 0}, {0, -4, 0}, {0, 0, 4}, {0, 0, -4},  // shell 6
    {1, 3, 3}, {-1, 3, 3}, {3, 1, 3}, {-3, 1, 3}, {3, -1, 3}, {-3, -1, 3}, {1, -3, 3},
    {-1, -3, 3}, {3, 3, 1}, {-3, 3, 1}, {3, -3, 1}, {-3, -3, 1}, {3, 3, -1}, {-3, 3, -1},
    {3, -3, -1}, {-3, -3, -1}, {1, 3, -3}, {-1, 3, -3}, {3, 1, -3}, {-3, 1, -3}, {3, -1, -3},
    {-3, -1, -3}, {1, -3, -3}, {-1, -3, -3},  // shell 7
    {0, 2, 4}, {2, 0, 4}, {-2, 0, 4}, {0, -2, 4}, {0, 4, 2}, {-4, 0, 2}, {4, 0, 2},
    {0, -4, 2}, {2, 4, 0}, {-2, 4, 0}, {4, 2, 0}, {-4, 2, 0}, {4, -2, 0}, {-4, -2, 0},
    {0, 4, 0}, {-4, 0, 0}, {0, 4, -2}, {-4, 0, -2}, {4, 0, -2}, {0, -4, -2}, {0, 2, -4},
    {2, 0, -4}, {-2, 0, -4}, {0, -2, -4},  // shell 8
    {2, 2, 4}, {-2, 2, 4}, {2, -2, 4}, {-2, -2, 4}, {2, 4, 2}, {-2, 4, 2}, {4, 2, 2},
    {-4, 2, 2}, {4, -2, 2}, {-4, -2, 2}, {2, -4, 2}, {-2, -4, 2}, {2, 4, -2}, {-2, 4, -2},
    {4, 2, -2}, {-4, 2, -2}, {4, -2, -2}, {-4, -2, -2}, {2, -4, -2}, {-2, -4, -2},
    {2, 2, -4}, {-2, 2, -4}, {2, -2, -4}, {-2, -2, -4},  // shell 9
    {1, 1, 5}, {-1, 1, 5}, {1, -1, 5}, {-1, -1, 5}, {3, 3, 3}, {-3, 3, 3}, {3, -3, 3},
    {-3, -3, 3}, {1, -5, 1}, {-1, -5, 1}, {5, -1, 1}, {-5, -1, 1}, {5, 1, 1}, {-5, 1, 1},
    {1, -5, 1}, {-1, -5, 1}, {1, -5, -1}, {-1, -5, -1}, {5, -1, -1}, {-5, -1, -1},
    {5, 1, -1}, {-5, 1, -1}, {1, -5, -1}, {-1, -5, -1}, {3, 3, -3}, {-3, 3, -3},
    {3, -3, -3}, {-3, -3, -3}, {1, 1, -5}, {-1, 1, -5}, {1, -1, -5}, {-1, -1, -5},  // shell 10
};
BRAWL_TABLE int16_t kBCCShellStart[11] = {0, 8, 14, 26, 50, 58, 64, 88, 112, 136, 168};

// fcc: 6 shells, 86 entries
BRAWL_TABLE int8_t kFCCOffsets[86][3] = {
    {0, -1, 1}, {0, -1, -1}, {0, 1, 1}, {0, 1, -1}, {1, -1, 0}, {1, 1, 0}, {1, 0, 1},
    {1, 0, -1}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, 1}, {-1, 0, -1},  // shell 1
    {2, 0, 0}, {-2, 0, 0}, {0, 2, 0}, {0, -2, 0}, {0, 0, 2}, {0, 0, -2},  // shell 2
    {-2, 1, 1}, {-2, 1, -1}, {-2, -1, 1}, {-2, -1, -1}, {2, 1, 1}, {2, 1, -1}, {2, -1, 1},
    {2, -1, -1}, {1, 2, 1}, {-1, 2, 1}, {1, 2, -1}, {-1, 2, -1}, {1, -2, 1}, {-1, -2, 1},
    {1, -2, -1}, {-1, -2, -1}, {1, 1, 2}, {-1, 1, 2}, {1, -1, 2}, {-1, -1, 2}, {1, 1, -2},
    {-1, 1, -2}, {1, -1, -2}, {-1, -1, -2},  // shell 3
    {2, 0, -2}, {-2, 0, -2}, {0, 2, -2}, {0, -2, -2}, {2, 2, 0}, {-2, 2, 0}, {2, -2, 0},
    {-2, -2, 0}, {2, 0, 2}, {-2, 0, 2}, {0, 2, 2}, {0, -2, 2},  // shell 4
    {1, 0, -3}, {-1, 0, -3}, {0, -1, -3}, {0, 1, -3}, {0, 3, -1}, {3, 0, -1}, {-3, 0, -1},
    {0, -3, -1}, {1, 3, 0}, {-1, 3, 0}, {3, 1, 0}, {-3, 1, 0}, {3, -1, 0}, {-3, -1, 0},
    {1, -3, 0}, {-1, -3, 0}, {0, 3, 1}, {3, 0, 1}, {-3, 0, 1}, {0, -3, 1}, {1, 0, 3},
    {-1, 0, 3}, {0, -1, 3}, {0, 1, 3},  // shell 5
    {2, 2, -2}, {-2, 2, -2}, {2, -2, -2}, {-2, -2, -2}, {2, 2, 2}, {-2, 2, 2}, {2, -2, 2},
    {-2, -2, 2},  // shell 6
};
BRAWL_TABLE int16_t kFCCShellStart[7] = {0, 12, 18, 42, 54, 78, 86};

// Nearest-neighbour vectors drawn by the nbr_swap proposals, in the order of
// the reference's sc_nbrs / bcc_nbrs / fcc_nbrs (src/random_site.f90:29-61).
BRAWL_TABLE int8_t kSCNbrSwap[6][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0},
                                       {0, 0, -1}, {0, -1, 0}, {-1, 0, 0}};
BRAWL_TABLE int8_t kBCCNbrSwap[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                        {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
BRAWL_TABLE int8_t kFCCNbrSwap[12][3] = {{0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
                                         {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1},
                                         {-1, 1, 0}, {-1, -1, 0}, {-1, 0, 1}, {-1, 0, -1}};

inline int max_shells(int lattice) {
  // src/initialise.F90:160-241
  return lattice == kSimpleCubic ? 2 : lattice == kBcc ? 10 : lattice == kFcc ? 6 : 0;
}

inline const int8_t (*shell_offsets(int lattice))[3] {
  return lattice == kSimpleCubic ? kSCOffsets : lattice == kBcc ? kBCCOffsets : kFCCOffsets;
}

inline const int16_t* shell_starts(int lattice) {
  return lattice == kSimpleCubic ? kSCShellStart : lattice == kBcc ? kBCCShellStart
                                                                   : kFCCShellStart;
}

// Occupied sites: src/initialise.F90:162,175,214.
inline int n_atoms(int lattice, int n1, int n2, int n3) {
  int f = lattice == kSimpleCubic ? 8 : lattice == kBcc ? 2 : 4;
  return f * n1 * n2 * n3;
}

}  // namespace brawl
