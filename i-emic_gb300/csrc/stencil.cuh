// Stencil metadata shared by host set-up code and device kernels.
//
// THCM couples the six unknowns of a cell (u,v,w,p,T,S; src/ocean/par.F90:72-77)
// to neighbours at the 27 stencil positions of src/ocean/assemble.F90:142-179
// (kk = 1..9 level k, 10..18 level k-1, 19..27 level k+1; inside a level
// j offset = mod(kk+2,3)-1, i offset = (kk-1 mod 9)/3-1).
//
// For every row type this file lists the (position, column unknown) pairs of
// the maximal Jacobian graph in the order src/ocean/THCM.C:2300-2580 inserts
// them ("canonical entries"). Every coefficient the Fortran physics can make
// nonzero lies in this list, so the GPU kernels keep one register per entry.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define IEMIC_HD __host__ __device__
#else
#define IEMIC_HD
#endif

namespace iemic {

enum Unknown { UU = 1, VV = 2, WW = 3, PP = 4, TT = 5, SS = 6 };
enum Mask { OCEAN = 0, LAND = 1, WATER = 2, PERIO = 3 };
constexpr int NUN = 6;
constexpr int NPAR = 30;
// par(1..30) indices, src/ocean/par.F90:41-70
enum Par {
    AL_T = 1, RAYL, EK_V, EK_H, ROSB, MIXP, RESC, SPL1, HMTP, SUNP, PE_H, PE_V, P_VC,
    LAMB, SALT, WIND, TEMP, BIOT, COMB, ARCL, NLES, IFRICB, CONT, ENER, ALPC, CMPR,
    FPER, SPER, MKAP, SPL2
};

struct Ent { int kk, B; };

// canonical entry lists per row type (A = 1..6), as constexpr functions so
// device code can index them at run time
IEMIC_HD constexpr Ent entry(int A, int e) {
    constexpr Ent LU[24] = {{5, UU}, {2, UU}, {8, UU}, {4, UU}, {6, UU}, {14, UU}, {23, UU},
                            {5, VV}, {2, VV}, {8, VV}, {4, VV}, {6, VV},
                            {5, WW}, {8, WW}, {9, WW}, {6, WW}, {14, WW}, {17, WW}, {18, WW}, {15, WW},
                            {5, PP}, {8, PP}, {6, PP}, {9, PP}};
    constexpr Ent LV[22] = {{5, VV}, {2, VV}, {8, VV}, {4, VV}, {6, VV}, {14, VV}, {23, VV},
                            {5, UU}, {2, UU}, {8, UU},
                            {5, WW}, {8, WW}, {9, WW}, {6, WW}, {14, WW}, {17, WW}, {18, WW}, {15, WW},
                            {5, PP}, {8, PP}, {6, PP}, {9, PP}};
    constexpr Ent LW[7] = {{5, WW}, {5, PP}, {23, PP}, {5, TT}, {23, TT}, {5, SS}, {23, SS}};
    constexpr Ent LP[11] = {{5, PP}, {5, UU}, {2, UU}, {4, UU}, {1, UU}, {5, VV}, {2, VV}, {4, VV}, {1, VV},
                            {5, WW}, {14, WW}};
    constexpr Ent LT[20] = {{5, TT}, {2, TT}, {8, TT}, {4, TT}, {6, TT}, {14, TT}, {23, TT},
                            {5, UU}, {2, UU}, {1, UU}, {4, UU}, {5, VV}, {2, VV}, {1, VV}, {4, VV},
                            {5, WW}, {14, WW}, {5, SS}, {14, SS}, {23, SS}};
    constexpr Ent LS[20] = {{5, SS}, {2, SS}, {8, SS}, {4, SS}, {6, SS}, {14, SS}, {23, SS},
                            {5, UU}, {2, UU}, {1, UU}, {4, UU}, {5, VV}, {2, VV}, {1, VV}, {4, VV},
                            {5, WW}, {14, WW}, {5, TT}, {14, TT}, {23, TT}};
    return A == UU ? LU[e] : A == VV ? LV[e] : A == WW ? LW[e] : A == PP ? LP[e] : A == TT ? LT[e] : LS[e];
}
IEMIC_HD constexpr int rowlen(int A) {
    return A == UU ? 24 : A == VV ? 22 : A == WW ? 7 : A == PP ? 11 : A == TT ? 20 : A == SS ? 20 : 0;
}
// offset of a row type in the 104-entry list of a cell
IEMIC_HD constexpr int rowoff(int A) {
    return A <= UU ? 0 : A == VV ? 24 : A == WW ? 46 : A == PP ? 53 : A == TT ? 64 : A == SS ? 84 : 104;
}
constexpr int CELL_ENTRIES = 104;
// row type of an entry in the 104-entry cell list
IEMIC_HD constexpr int row_of_cell_entry(int e) {
    return e < 24 ? UU : e < 46 ? VV : e < 53 ? WW : e < 64 ? PP : e < 84 ? TT : SS;
}

// index of (kk, B) in the list of row type A, or -1
IEMIC_HD constexpr int idx(int A, int kk, int B) {
    for (int e = 0; e < rowlen(A); ++e)
        if (entry(A, e).kk == kk && entry(A, e).B == B) return e;
    return -1;
}
IEMIC_HD constexpr int dk_of(int kk) { return kk < 10 ? 0 : (kk < 19 ? -1 : 1); }
IEMIC_HD constexpr int dj_of(int kk) { return (kk + 2) % 3 - 1; }
IEMIC_HD constexpr int di_of(int kk) { return ((kk - 1) % 9) / 3 - 1; }

// rank of entry e of row type A in ascending (kk, B) order: the order in
// which src/ocean/assemble.F90 fillcolA emits a row, and hence the order in
// which src/ocean/matetc.F90 matAvec accumulates it.
IEMIC_HD constexpr int fortran_rank(int A, int e) {
    int r = 0;
    Ent x = entry(A, e);
    for (int q = 0; q < rowlen(A); ++q) {
        Ent y = entry(A, q);
        if (y.kk < x.kk || (y.kk == x.kk && y.B < x.B)) ++r;
    }
    return r;
}

// Boundary class of a cell: bit0 = first index, bit1 = last index, per axis.
IEMIC_HD inline int axis_class(int i, int n) { return (i == 0 ? 1 : 0) | (i == n - 1 ? 2 : 0); }
IEMIC_HD inline int cell_class(int i, int j, int k, int n, int m, int l) {
    return axis_class(i, n) | (axis_class(j, m) << 2) | (axis_class(k, l) << 4);
}
constexpr int NCLASS = 64;

// compile-time loop helper
template <int N>
struct IC { static constexpr int value = N; };
template <int B, int E, class F>
IEMIC_HD inline void static_for(F&& f) {
    if constexpr (B < E) {
        f(IC<B>{});
        static_for<B + 1, E>(f);
    }
}

}  // namespace iemic
