// Deterministic colouring of the solver list (host side of the library).
//
// Nodes are solver updateables in list order (joints, then manifolds); two
// updateables conflict when they share a dynamic body -- the only bodies the
// reference locks (SolverUpdateable.cs:151-160).  Greedy first-fit in list
// order gives every updateable the smallest colour unused at its dynamic
// bodies; the colour-sorted order is stable (list order inside a colour).
// Within a colour no two updateables touch the same dynamic body, so a colour
// is one data-parallel Gauss-Seidel sweep whose result equals the sequential
// sweep over the same members.
#pragma once
#include <cstdint>
#include <vector>

namespace bepugpu {

struct Colouring {
    std::vector<int32_t> colour;   // per updateable
    std::vector<int32_t> order;    // colour-sorted list of updateables
    std::vector<int32_t> offsets;  // order[offsets[c] .. offsets[c+1]) have colour c
    int32_t colours = 0;
};

// a[i], b[i]: body indices of updateable i (-1 = none); dynamic[k] != 0 for
// dynamic bodies.  follows[i] != 0 (null: none) marks an entry that is part of
// entry i - 1's visit (a group's continuation record): it takes i - 1's colour
// and claims nothing, so the rest of the colouring is the one of the list
// without it.  Returns false if an index is out of range.
bool ColourSolverList(const int32_t* a, const int32_t* b, int32_t n, const uint8_t* dynamic, int32_t bodies,
                      Colouring& out, const uint8_t* follows = nullptr);

}  // namespace bepugpu
