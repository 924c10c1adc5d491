// fit_kernels.cuh -- device code of the FIT leapfrog path for sm_103a.
//
// Field layout (shared with the Python Field class): a field is 3*N values, component
// blocks [x | y | z], each block in Fortran order n = i + Nx*j + Nx*Ny*k.  The curl is
// the reference's sparse matrix C (wakis/solverFIT3D.py:207-227) applied matrix-free:
// forward differences D_a v[n] = v[n+s_a] - v[n] with v[n+s_a] = 0 past the end of the
// block, and backward differences for C^T.  Neighbours follow the FLAT index, so at
// i = Nx-1 the x neighbour of (i, j, k) is (0, j+1, k) and at j = Ny-1 the y neighbour
// is (i, 0, k+1); the face masks zero those couplings for PEC/PML faces and leave them
// live for periodic / ABC / open faces, exactly as the matrix does.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "wakis_fit.h"

namespace fit {

// Unsigned 32-bit division by an invariant divisor d with one multiply-high
// (Granlund & Montgomery, "Division by invariant integers using multiplication", 1994,
// Fig. 4.1): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// q = (t + ((n - t) >> min(l,1))) >> max(l-1,0) with t = mulhi(m, n); exact for n < 2^32.
struct FastDiv {
    unsigned d, m;
    int s1, s2;
};

inline FastDiv make_fastdiv(unsigned d) {
    int l = 0;
    while ((1ull << l) < d) ++l;
    FastDiv f;
    f.d = d;
    f.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l - 1 > 0 ? l - 1 : 0;
    return f;
}

__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv& f) {
    const unsigned t = __umulhi(f.m, n);
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

// face bit f: 0 x-lo, 1 x-hi, 2 y-lo, 3 y-hi, 4 z-lo, 5 z-hi
struct Geom {
    int nx, ny, nz;
    int pad;
    long long N;   // cells per component
    long long sy;  // Nx
    long long sz;  // Nx*Ny
    unsigned pec;  // faces whose tangential E columns are zeroed (Dbc of PEC/PML)
    unsigned pmc;  // faces whose tangential H rows/columns are zeroed (Dbc of PMC)
    FastDiv fx, fy;  // division by Nx and by Ny
};

// A thread's VEC cells (i0..i0+VEC-1, j, k) and all their +-1 neighbours lie at least one
// cell away from every face: no face mask, no row crossing, no truncation applies.
template <int VEC>
__device__ __forceinline__ bool interior(int i0, int j, int k, const Geom& g) {
    return i0 >= 2 && i0 + VEC + 2 <= g.nx && j >= 2 && j + 3 <= g.ny && k >= 2 && k + 3 <= g.nz;
}

// Row (j, k) at least two cells from the y and z faces: neighbours along y and z stay in
// the block, no y/z face mask applies, and the only row crossing is the x one.  All
// threads of a warp share one row on grids with Nx >= 32*VEC, so this test does not
// split warps there.
__device__ __forceinline__ bool row_interior(int j, int k, const Geom& g) {
    return j >= 2 && j + 3 <= g.ny && k >= 2 && k + 3 <= g.nz;
}

// Dbc face mask of component d at (i, j, k).  The reference writes the mask plane by
// plane in the order x-lo, x-hi, y-lo, y-hi, z-lo, z-hi skipping the component's own
// axis, so the LAST applicable write wins (wakis/boundaries.py:92-101): test in
// reverse order.
__device__ __forceinline__ bool face_open(unsigned bits, int d, int i, int j, int k, const Geom& g) {
    if (bits == 0u) return true;
    if (d != 2) {
        if (k == g.nz - 1) return !((bits >> 5) & 1u);
        if (k == 0) return !((bits >> 4) & 1u);
    }
    if (d != 1) {
        if (j == g.ny - 1) return !((bits >> 3) & 1u);
        if (j == 0) return !((bits >> 2) & 1u);
    }
    if (d != 0) {
        if (i == g.nx - 1) return !((bits >> 1) & 1u);
        if (i == 0) return !(bits & 1u);
    }
    return true;
}

template <typename T>
struct Metric {
    const T* L[3];   // primal edge lengths dx[i], dy[j], dz[k]
    const T* tL[3];  // dual edge lengths after the periodic / ABC edits
};

// coordinate of a flat neighbour (flat-index semantics; valid = inside the block)
struct Nb {
    int i, j, k;
    bool valid;
};

__device__ __forceinline__ Nb fwd_x(int i, int j, int k, const Geom& g) {
    if (i + 1 < g.nx) return {i + 1, j, k, true};
    if (j + 1 < g.ny) return {0, j + 1, k, true};
    if (k + 1 < g.nz) return {0, 0, k + 1, true};
    return {0, 0, 0, false};
}
__device__ __forceinline__ Nb fwd_y(int i, int j, int k, const Geom& g) {
    if (j + 1 < g.ny) return {i, j + 1, k, true};
    if (k + 1 < g.nz) return {i, 0, k + 1, true};
    return {0, 0, 0, false};
}
__device__ __forceinline__ Nb fwd_z(int i, int j, int k, const Geom& g) {
    if (k + 1 < g.nz) return {i, j, k + 1, true};
    return {0, 0, 0, false};
}
__device__ __forceinline__ Nb bwd_x(int i, int j, int k, const Geom& g) {
    if (i > 0) return {i - 1, j, k, true};
    if (j > 0) return {g.nx - 1, j - 1, k, true};
    if (k > 0) return {g.nx - 1, g.ny - 1, k - 1, true};
    return {0, 0, 0, false};
}
__device__ __forceinline__ Nb bwd_y(int i, int j, int k, const Geom& g) {
    if (j > 0) return {i, j - 1, k, true};
    if (k > 0) return {i, g.ny - 1, k - 1, true};
    return {0, 0, 0, false};
}
__device__ __forceinline__ Nb bwd_z(int i, int j, int k, const Geom& g) {
    if (k > 0) return {i, j, k - 1, true};
    return {0, 0, 0, false};
}

template <typename T>
__device__ __forceinline__ T edge_len(const T* const* L, int d, int i, int j, int k) {
    return d == 0 ? L[0][i] : (d == 1 ? L[1][j] : L[2][k]);
}

// Explicitly rounded arithmetic of the stencils: one rounding per multiply, add and
// fused multiply-add, in a fixed pattern.  Every kernel that inlines the stencil
// functions (fused or two-pass, coded or dense coefficients) then computes the same bits,
// whatever multiply-adds the compiler would have contracted in each of them.
template <typename T>
__device__ __forceinline__ T rmul(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fmul_rn(a, b);
    else return __dmul_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T radd(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fadd_rn(a, b);
    else return __dadd_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T rsub(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fsub_rn(a, b);
    else return __dsub_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T rfma(T a, T b, T c) {  // a*b + c
    if constexpr (sizeof(T) == 4) return __fmaf_rn(a, b, c);
    else return __fma_rn(a, b, c);
}

// ê_d(m) = Dbc_pec * L_d * E_d[m]  (column scaling of C by Ds and Dbc)
template <typename T>
__device__ __forceinline__ T ehat(T e, int d, const Nb& p, const Geom& g, const Metric<T>& m) {
    if (!p.valid) return T(0);
    if (!face_open(g.pec, d, p.i, p.j, p.k, g)) return T(0);
    return rmul(edge_len<T>(m.L, d, p.i, p.j, p.k), e);
}
// ĥ_d(m) = Dbc_pmc * tL_d * H_d[m]
template <typename T>
__device__ __forceinline__ T hhat(T h, int d, const Nb& p, const Geom& g, const Metric<T>& m) {
    if (!p.valid) return T(0);
    if (!face_open(g.pmc, d, p.i, p.j, p.k, g)) return T(0);
    return rmul(edge_len<T>(m.tL, d, p.i, p.j, p.k), h);
}

// ---------------------------------------------------------------- vector loads/stores
// a hint that the line holding p will be read soon: fetched into L2, nothing waits on it
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
template <typename T, int VEC>
__device__ __forceinline__ void ldg_v(T (&r)[VEC], const T* __restrict__ p) {
    if constexpr (VEC == 4 && sizeof(T) == 4) {
        float4 t = __ldg(reinterpret_cast<const float4*>(p));
        r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
    } else if constexpr (VEC == 2 && sizeof(T) == 8) {
        double2 t = __ldg(reinterpret_cast<const double2*>(p));
        r[0] = t.x; r[1] = t.y;
    } else if constexpr (VEC == 2 && sizeof(T) == 4) {
        float2 t = __ldg(reinterpret_cast<const float2*>(p));
        r[0] = t.x; r[1] = t.y;
    } else {
#pragma unroll
        for (int e = 0; e < VEC; ++e) r[e] = __ldg(p + e);
    }
}
template <typename T, int VEC>
__device__ __forceinline__ void ld_v(T (&r)[VEC], const T* p) {
    if constexpr (VEC == 4 && sizeof(T) == 4) {
        float4 t = *reinterpret_cast<const float4*>(p);
        r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
    } else if constexpr (VEC == 2 && sizeof(T) == 8) {
        double2 t = *reinterpret_cast<const double2*>(p);
        r[0] = t.x; r[1] = t.y;
    } else if constexpr (VEC == 2 && sizeof(T) == 4) {
        float2 t = *reinterpret_cast<const float2*>(p);
        r[0] = t.x; r[1] = t.y;
    } else {
#pragma unroll
        for (int e = 0; e < VEC; ++e) r[e] = p[e];
    }
}
template <typename T, int VEC>
__device__ __forceinline__ void st_v(T* p, const T (&r)[VEC]) {
    if constexpr (VEC == 4 && sizeof(T) == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
    } else if constexpr (VEC == 2 && sizeof(T) == 8) {
        *reinterpret_cast<double2*>(p) = make_double2(r[0], r[1]);
    } else if constexpr (VEC == 2 && sizeof(T) == 4) {
        *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
    } else {
#pragma unroll
        for (int e = 0; e < VEC; ++e) p[e] = r[e];
    }
}
template <typename T, int VEC>
__device__ __forceinline__ void zero_v(T (&r)[VEC]) {
#pragma unroll
    for (int e = 0; e < VEC; ++e) r[e] = T(0);
}

// ---------------------------------------------------------------- coded coefficients
// A grid has few distinct per-cell coefficient triples (ch, ce, cl): uniform spacing,
// a handful of materials, graded PML planes.  A coded context stores one 16-bit code
// per cell and a table tab[code][group][4] (group 0 ch, 1 ce, 2 cl; x, y, z, pad) that
// holds the exact values of the dense arrays, so a coded step gives the dense step's
// results bit for bit while reading 2 bytes instead of 9 words per cell.
template <int VEC>
__device__ __forceinline__ void ld_codes(unsigned (&c)[VEC], const unsigned short* __restrict__ p) {
    if constexpr (VEC == 4) {
        const uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
        c[0] = t.x & 0xffffu; c[1] = t.x >> 16; c[2] = t.y & 0xffffu; c[3] = t.y >> 16;
    } else if constexpr (VEC == 2) {
        const unsigned t = __ldg(reinterpret_cast<const unsigned*>(p));
        c[0] = t & 0xffffu; c[1] = t >> 16;
    } else {
#pragma unroll
        for (int e = 0; e < VEC; ++e) c[e] = __ldg(p + e);
    }
}
template <typename T>
__device__ __forceinline__ void tab_get(const T* __restrict__ tab, unsigned code, int grp, T& x, T& y, T& z) {
    if constexpr (sizeof(T) == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(tab) + 3 * code + grp);
        x = t.x; y = t.y; z = t.z;
    } else {
        const double2* q = reinterpret_cast<const double2*>(tab) + 2 * (3 * code + grp);
        const double2 a = __ldg(q), b = __ldg(q + 1);
        x = a.x; y = a.y; z = b.x;
    }
}
// the VEC cells of a thread mostly share one code (material boundaries are rare): one
// table read then serves all of them
template <typename T, int VEC>
__device__ __forceinline__ void tab_get_v(const T* __restrict__ tab, const unsigned (&c)[VEC], int grp, T (&x)[VEC],
                                          T (&y)[VEC], T (&z)[VEC]) {
    bool same = true;
#pragma unroll
    for (int e = 1; e < VEC; ++e) same = same && c[e] == c[0];
    if (same) {
        T a, b, d;
        tab_get<T>(tab, c[0], grp, a, b, d);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            x[e] = a;
            y[e] = b;
            z[e] = d;
        }
    } else {
#pragma unroll
        for (int e = 0; e < VEC; ++e) tab_get<T>(tab, c[e], grp, x[e], y[e], z[e]);
    }
}

// ---------------------------------------------------------------- beam line current
// sources.Beam.update (wakis/sources.py:98-110), evaluated in FP64 with the reference's
// operation order:  J = ((q*v)*profile)/dx/dy,
//   profile = (1/sqrt(2*pi*sigmaz^2)) * exp(-((z - vt) - s0)^2 / (2*sigmaz^2)).
struct BeamArgs {
    int active;
    int ixs, iys;
    double qv;        // q*v
    double c0;        // 1/sqrt(2*pi*sigmaz^2)
    double two_s2;    // 2*sigmaz^2
    double s0;        // zmin - v*ti
    double dx_s, dy_s;
    const double* z;  // cell-centre z, nz values
    const double* dtieps;  // dt*ieps_z on the line, nz values (FP64)
};

__device__ __forceinline__ double beam_current(const BeamArgs& b, int k, double vt) {
    double s = __dsub_rn(b.z[k], vt);
    double d = __dsub_rn(s, b.s0);
    double prof = __dmul_rn(b.c0, exp(-__dmul_rn(d, d) / b.two_s2));
    return __dmul_rn(b.qv, prof) / b.dx_s / b.dy_s;
}

// step number / beam position of a launch: host-driven launches pass them as values;
// graph-replayed launches read the step counter on the device.
struct StepArgs {
    long long n;
    double vt;
    const long long* d_step;  // if set: n = *d_step - 1 (the prologue already advanced it)
    const double* vt_table;   // with d_step: vt = vt_table[n]
    long long vt_len;
};

__device__ __forceinline__ void resolve_step(const StepArgs& s, long long& n, double& vt) {
    if (s.d_step) {
        n = *s.d_step - 1;
        vt = (s.vt_table && n >= 0 && n < s.vt_len) ? s.vt_table[n] : 0.0;
    } else {
        n = s.n;
        vt = s.vt;
    }
}

struct PlaneArgs {
    int active;
    int zs, x0, x1, y0, y1;
    const double* prof;  // (x1-x0)*(y1-y0) or null
    const double* c1;
    const double* c2;
    const double* gt;
    long long len;
    double* stash;  // E_x of the plane before the source overwrote it (loss term)
};

// ---------------------------------------------------------------- pass arithmetic
// One thread updates VEC consecutive x cells (i0..i0+VEC-1, j, k).  The inputs are the
// VEC values of each stream at the thread's cells (own, +Nx row, +Nx*Ny plane) and the
// one value just past the vector along x; they come from registers (direct kernels)
// or from shared memory (staged kernels).

// H_c <- H_c - ch_c * (C ê)_c
template <typename T, int VEC>
__device__ __forceinline__ void hpass_cells(const T (&ex)[VEC], const T (&ey)[VEC], const T (&ez)[VEC],
                                            const T (&exy)[VEC], const T (&ezy)[VEC], const T (&exz)[VEC],
                                            const T (&eyz)[VEC], T eyx, T ezx, T (&hx)[VEC], T (&hy)[VEC],
                                            T (&hz)[VEC], const T (&cx)[VEC], const T (&cy)[VEC],
                                            const T (&cz)[VEC], int i0, int j, int k, const Geom& g,
                                            const Metric<T>& mt) {
    if (row_interior(j, k, g)) {
        // j and k at least 2 cells from the y / z faces: the only masks are those of the
        // x faces on the y, z components, and the only crossing is the x neighbour of
        // i = Nx-1, which is (0, j+1, k).  Edge lengths: L_x(i), L_y(j), L_z(k).
        const T ly = mt.L[1][j], lz = mt.L[2][k];
        const bool xlo = g.pec & 1u, xhi = (g.pec >> 1) & 1u;
        const int il = i0 + VEC;
        const bool cross = il >= g.nx;
        const T mlast = cross ? (xlo ? T(0) : T(1)) : (((il == g.nx - 1) && xhi) ? T(0) : T(1));
        const T lyl = cross ? mt.L[1][j + 1] : ly;
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int i = i0 + e;
            const T lx = mt.L[0][i];
            const T me = (((i == 0) && xlo) || ((i == g.nx - 1) && xhi)) ? T(0) : T(1);
            const T mn = (e + 1 < VEC) ? ((((i + 1) == g.nx - 1) && xhi) ? T(0) : T(1)) : mlast;
            const T lyn = (e + 1 < VEC) ? ly : lyl;
            const T eyX = (e + 1 < VEC) ? ey[e + 1] : eyx;
            const T ezX = (e + 1 < VEC) ? ez[e + 1] : ezx;
            const T curlx = rmul(me, rfma(ly, rsub(ey[e], eyz[e]), rmul(lz, rsub(ezy[e], ez[e]))));
            const T curly = rfma(lx, rsub(exz[e], ex[e]), rmul(lz, rfma(me, ez[e], -rmul(mn, ezX))));
            const T curlz = rfma(lx, rsub(ex[e], exy[e]), rfma(rmul(mn, lyn), eyX, -rmul(rmul(me, ly), ey[e])));
            hx[e] = rfma(-cx[e], curlx, hx[e]);
            hy[e] = rfma(-cy[e], curly, hy[e]);
            hz[e] = rfma(-cz[e], curlz, hz[e]);
        }
        return;
    }
    const Nb xl = fwd_x(i0 + VEC - 1, j, k, g);
    const Nb py = fwd_y(i0, j, k, g);
    const Nb pz = fwd_z(i0, j, k, g);
#pragma unroll
    for (int e = 0; e < VEC; ++e) {
        const int i = i0 + e;
        const Nb p0{i, j, k, true};
        const Nb pyi{i, py.j, py.k, py.valid};
        const Nb pzi{i, pz.j, pz.k, pz.valid};
        const Nb pxi = (e + 1 < VEC) ? Nb{i + 1, j, k, true} : xl;
        const T ex0 = ehat<T>(ex[e], 0, p0, g, mt);
        const T ey0 = ehat<T>(ey[e], 1, p0, g, mt);
        const T ez0 = ehat<T>(ez[e], 2, p0, g, mt);
        const T exY = ehat<T>(exy[e], 0, pyi, g, mt);
        const T ezY = ehat<T>(ezy[e], 2, pyi, g, mt);
        const T exZ = ehat<T>(exz[e], 0, pzi, g, mt);
        const T eyZ = ehat<T>(eyz[e], 1, pzi, g, mt);
        const T eyX = ehat<T>((e + 1 < VEC) ? ey[e + 1] : eyx, 1, pxi, g, mt);
        const T ezX = ehat<T>((e + 1 < VEC) ? ez[e + 1] : ezx, 2, pxi, g, mt);
        // (C ê)_x = -D_z ê_y + D_y ê_z ; (C ê)_y = D_z ê_x - D_x ê_z ; (C ê)_z = -D_y ê_x + D_x ê_y
        const T curlx = radd(rsub(ey0, eyZ), rsub(ezY, ez0));
        const T curly = radd(rsub(exZ, ex0), rsub(ez0, ezX));
        const T curlz = radd(rsub(ex0, exY), rsub(eyX, ey0));
        hx[e] = rfma(-cx[e], curlx, hx[e]);
        hy[e] = rfma(-cy[e], curly, hy[e]);
        hz[e] = rfma(-cz[e], curlz, hz[e]);
    }
}

// (C^T ĥ)_c of VEC cells, D^T_a v[m] = v[m - s_a] - v[m]
template <typename T, int VEC>
__device__ __forceinline__ void epass_curl(const T (&hx)[VEC], const T (&hy)[VEC], const T (&hz)[VEC],
                                           const T (&hxy)[VEC], const T (&hzy)[VEC], const T (&hxz)[VEC],
                                           const T (&hyz)[VEC], T hyx, T hzx, T (&cur)[3][VEC], int i0, int j,
                                           int k, const Geom& g, const Metric<T>& mt) {
    if (row_interior(j, k, g)) {
        // PMC masks of the x faces on the y, z components; the x neighbour of i = 0 is
        // (Nx-1, j-1, k).  Dual lengths: tL_x(i), tL_y(j), tL_z(k).
        const T ly = mt.tL[1][j], lz = mt.tL[2][k];
        const bool plo = g.pmc & 1u, phi = (g.pmc >> 1) & 1u;
        const bool cross = i0 == 0;
        const T mfirst = cross ? (phi ? T(0) : T(1)) : ((((i0 - 1) == 0) && plo) ? T(0) : T(1));
        const T lyf = cross ? mt.tL[1][j - 1] : ly;
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int i = i0 + e;
            const T lx = mt.tL[0][i];
            const T mpe = (((i == 0) && plo) || ((i == g.nx - 1) && phi)) ? T(0) : T(1);
            const T mpp = (e > 0) ? ((((i - 1) == 0) && plo) ? T(0) : T(1)) : mfirst;
            const T lyp = (e > 0) ? ly : lyf;
            const T hyX = (e > 0) ? hy[e - 1] : hyx;
            const T hzX = (e > 0) ? hz[e - 1] : hzx;
            cur[0][e] = rmul(mpe, rfma(ly, rsub(hyz[e], hy[e]), rmul(lz, rsub(hz[e], hzy[e]))));
            cur[1][e] = rfma(lx, rsub(hx[e], hxz[e]), rmul(lz, rfma(mpp, hzX, -rmul(mpe, hz[e]))));
            cur[2][e] = rfma(lx, rsub(hxy[e], hx[e]), rfma(rmul(mpe, ly), hy[e], -rmul(rmul(mpp, lyp), hyX)));
        }
        return;
    }
    const Nb xf = bwd_x(i0, j, k, g);
    const Nb py = bwd_y(i0, j, k, g);
    const Nb pz = bwd_z(i0, j, k, g);
#pragma unroll
    for (int e = 0; e < VEC; ++e) {
        const int i = i0 + e;
        const Nb p0{i, j, k, true};
        const Nb pyi{i, py.j, py.k, py.valid};
        const Nb pzi{i, pz.j, pz.k, pz.valid};
        const Nb pxi = (e > 0) ? Nb{i - 1, j, k, true} : xf;
        const T hx0 = hhat<T>(hx[e], 0, p0, g, mt);
        const T hy0 = hhat<T>(hy[e], 1, p0, g, mt);
        const T hz0 = hhat<T>(hz[e], 2, p0, g, mt);
        const T hxY = hhat<T>(hxy[e], 0, pyi, g, mt);
        const T hzY = hhat<T>(hzy[e], 2, pyi, g, mt);
        const T hxZ = hhat<T>(hxz[e], 0, pzi, g, mt);
        const T hyZ = hhat<T>(hyz[e], 1, pzi, g, mt);
        const T hyX = hhat<T>((e > 0) ? hy[e - 1] : hyx, 1, pxi, g, mt);
        const T hzX = hhat<T>((e > 0) ? hz[e - 1] : hzx, 2, pxi, g, mt);
        // (C^T ĥ)_x = D^T_z ĥ_y - D^T_y ĥ_z ; (C^T ĥ)_y = -D^T_z ĥ_x + D^T_x ĥ_z ;
        // (C^T ĥ)_z = D^T_y ĥ_x - D^T_x ĥ_y
        cur[0][e] = radd(rsub(hyZ, hy0), rsub(hz0, hzY));
        cur[1][e] = radd(rsub(hx0, hxZ), rsub(hzX, hz0));
        cur[2][e] = radd(rsub(hxY, hx0), rsub(hy0, hyX));
    }
}

// Elided-J E update of VEC cells (MODE 0: no conduction current, MODE 1: loss factor),
// with the beam line current and the hard-source plane (stash) corrections.
template <typename T, int VEC, int MODE>
__device__ __forceinline__ void epass_update(T (&ex)[VEC], T (&ey)[VEC], T (&ez)[VEC], const T (&kx)[VEC],
                                             const T (&ky)[VEC], const T (&kz)[VEC], const T (&lx)[VEC],
                                             const T (&ly)[VEC], const T (&lz)[VEC], const T (&cur)[3][VEC],
                                             T* __restrict__ J, long long n, int i0, int j, int k, int use_cond,
                                             const Geom& g, const BeamArgs& b, const PlaneArgs& pl,
                                             const StepArgs& st) {
    const bool on_line = b.active && (j == b.iys) && (b.ixs >= i0) && (b.ixs < i0 + VEC);
    double jb = 0.0;
    if (on_line) {
        long long sn;
        double vt;
        resolve_step(st, sn, vt);
        jb = beam_current(b, k, vt);
    }
    if constexpr (MODE == 0) {
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            ex[e] = rfma(kx[e], cur[0][e], ex[e]);
            ey[e] = rfma(ky[e], cur[1][e], ey[e]);
            ez[e] = rfma(kz[e], cur[2][e], ez[e]);
        }
    } else {
        // on the hard-source plane the conduction current is sigma times the E_x the
        // source overwrote (J was computed at the end of the previous step)
        const bool on_plane = pl.active && k == pl.zs && j >= pl.y0 && j < pl.y1;
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int i = i0 + e;
            if (on_plane && i >= pl.x0 && i < pl.x1)
                ex[e] = rfma(kx[e], cur[0][e],
                             rsub(ex[e], rmul(rsub(T(1), lx[e]),
                                              (T)pl.stash[(i - pl.x0) + (j - pl.y0) * (pl.x1 - pl.x0)])));
            else
                ex[e] = rfma(kx[e], cur[0][e], rmul(lx[e], ex[e]));
            ey[e] = rfma(ky[e], cur[1][e], rmul(ly[e], ey[e]));
            // on the beam line J was overwritten by the beam: no sigma*E term there
            ez[e] = rfma(kz[e], cur[2][e], (on_line && (i0 + e == b.ixs)) ? ez[e] : rmul(lz[e], ez[e]));
        }
    }
    if (on_line) {
        const T dj = rmul((T)b.dtieps[k], (T)jb);
#pragma unroll
        for (int e = 0; e < VEC; ++e)
            if (i0 + e == b.ixs) ez[e] = rsub(ez[e], dj);
        if (!use_cond) J[2 * g.N + n + (b.ixs - i0)] = (T)jb;  // J keeps the last beam value
    }
}

// (i, j, k) of the component-local flat index n (N < 2^31 is checked on the host)
__device__ __forceinline__ void cell_of(long long n, const Geom& g, int& i0, int& j, int& k) {
    const unsigned u = (unsigned)n;
    const unsigned r = fdiv(u, g.fx);
    i0 = (int)(u - r * (unsigned)g.nx);
    const unsigned q = fdiv(r, g.fy);
    j = (int)(r - q * (unsigned)g.ny);
    k = (int)q;
}

// ---------------------------------------------------------------- direct kernels
// One thread per VEC cells, inputs loaded straight from global memory.  Used for grids
// whose Nx is not a multiple of the 16-byte vector width and for the explicit-J pass.
// New H of the VEC cells starting at component-local flat index n (cell (i0, j, k)),
// from E and the old H: the values land in hx, hy, hz; nothing is stored.
template <typename T, int VEC, bool CODED = false>
__device__ __forceinline__ void hpass_eval(const T* __restrict__ E, const T* H, const T* __restrict__ ch,
                                           const Geom& g, const Metric<T>& mt, long long n, int i0, int j, int k,
                                           T (&hx)[VEC], T (&hy)[VEC], T (&hz)[VEC],
                                           const unsigned short* __restrict__ code = nullptr,
                                           const T* __restrict__ tab = nullptr, const unsigned* pre = nullptr) {
    // 32-bit offsets from per-component pointers (n + Nx*Ny < 2^31 is checked on the
    // host): one multiply-add per address instead of 64-bit index arithmetic
    const int ni = (int)n, N = (int)g.N, sy = (int)g.sy, sz = (int)g.sz;
    const T* Ex = E + ni;
    const T* Ey = Ex + N;
    const T* Ez = Ey + N;
    T ex[VEC], ey[VEC], ez[VEC];
    ldg_v<T, VEC>(ex, Ex);
    ldg_v<T, VEC>(ey, Ey);
    ldg_v<T, VEC>(ez, Ez);
    const bool yv = (j + 1 < g.ny) || (k + 1 < g.nz);
    const bool zv = (k + 1 < g.nz);
    T exy[VEC], ezy[VEC], exz[VEC], eyz[VEC];
    if (yv) {
        ldg_v<T, VEC>(exy, Ex + sy);
        ldg_v<T, VEC>(ezy, Ez + sy);
    } else {
        zero_v<T, VEC>(exy);
        zero_v<T, VEC>(ezy);
    }
    if (zv) {
        ldg_v<T, VEC>(exz, Ex + sz);
        ldg_v<T, VEC>(eyz, Ey + sz);
    } else {
        zero_v<T, VEC>(exz);
        zero_v<T, VEC>(eyz);
    }
    T eyx = T(0), ezx = T(0);
    if (ni + VEC < N) {
        eyx = __ldg(Ey + VEC);
        ezx = __ldg(Ez + VEC);
    }
    T cx[VEC], cy[VEC], cz[VEC];
    const T* Hn = H + ni;
    ld_v<T, VEC>(hx, Hn);
    ld_v<T, VEC>(hy, Hn + N);
    ld_v<T, VEC>(hz, Hn + N + N);
    if constexpr (CODED) {
        unsigned cd[VEC];
        if (pre) {
#pragma unroll
            for (int e = 0; e < VEC; ++e) cd[e] = pre[e];
        } else {
            ld_codes<VEC>(cd, code + ni);
        }
        tab_get_v<T, VEC>(tab, cd, 0, cx, cy, cz);
    } else {
        const T* cn = ch + ni;
        ldg_v<T, VEC>(cx, cn);
        ldg_v<T, VEC>(cy, cn + N);
        ldg_v<T, VEC>(cz, cn + N + N);
    }
    hpass_cells<T, VEC>(ex, ey, ez, exy, ezy, exz, eyz, eyx, ezx, hx, hy, hz, cx, cy, cz, i0, j, k, g, mt);
}

// H pass of the VEC cells starting at component-local flat index n
template <typename T, int VEC, bool CODED = false>
__device__ __forceinline__ void hpass_at(const T* __restrict__ E, T* __restrict__ H, const T* __restrict__ ch,
                                         const Geom& g, const Metric<T>& mt, long long n,
                                         const unsigned short* __restrict__ code = nullptr,
                                         const T* __restrict__ tab = nullptr) {
    int i0, j, k;
    cell_of(n, g, i0, j, k);
    T hx[VEC], hy[VEC], hz[VEC];
    hpass_eval<T, VEC, CODED>(E, H, ch, g, mt, n, i0, j, k, hx, hy, hz, code, tab);
    st_v<T, VEC>(H + n, hx);
    st_v<T, VEC>(H + g.N + n, hy);
    st_v<T, VEC>(H + 2 * g.N + n, hz);
}

template <typename T, int VEC>
__global__ void __launch_bounds__(256, 3) k_hpass(const T* __restrict__ E, T* __restrict__ H,
                                               const T* __restrict__ ch, Geom g, Metric<T> mt) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.N / VEC) return;
    hpass_at<T, VEC>(E, H, ch, g, mt, v * VEC);
}

// the H pass with coded coefficients (ch from the code table).  ahead > 0: the thread
// first asks L2 for E, H and the code of the vector `ahead` vectors on, the one a thread
// of the next resident wave of CTAs works on.
template <typename T, int VEC>
__global__ void __launch_bounds__(256, 3) k_hpass_coded(const T* __restrict__ E, T* __restrict__ H, Geom g,
                                                     Metric<T> mt, const unsigned short* __restrict__ code,
                                                     const T* __restrict__ tab, long long ahead) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.N / VEC) return;
    if (ahead > 0 && (v + ahead) * VEC < g.N) {
        const long long m = (v + ahead) * VEC;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            prefetch_l2(E + c * g.N + m);
            prefetch_l2(H + c * g.N + m);
        }
        prefetch_l2(code + m);
    }
    hpass_at<T, VEC, true>(E, H, nullptr, g, mt, v * VEC, code, tab);
}

// MODE 0: E += ce*(C^T ĥ)                       (no conduction current)
// MODE 1: E = cl*E + ce*(C^T ĥ)                 (J = sigma*E_prev folded into cl)
// MODE 2: E = E + ce*(C^T ĥ) - cj*J; J = sg*E   (explicit J; J written if conductive)
// The beam line (ixs, iys, :) of the z component uses the beam current instead of J.
// E update of the VEC cells at flat index n (cell (i0, j, k)) from the new H around
// them: own (hx, hy, hz), the row below (hxy, hzy at n - Nx), the plane below (hxz, hyz
// at n - Nx*Ny) and the value before the vector along x (hyx, hzx at n - 1).  E is read
// from Esrc and written to Edst (the same array for the in-place passes).
// CODED (MODE 0 and 1): ce and cl come from the code table (code, tab)
template <typename T, int VEC, int MODE, bool CODED = false>
__device__ __forceinline__ void epass_finish(const T* Esrc, T* Edst, const T (&hx)[VEC], const T (&hy)[VEC],
                                             const T (&hz)[VEC], const T (&hxy)[VEC], const T (&hzy)[VEC],
                                             const T (&hxz)[VEC], const T (&hyz)[VEC], T hyx, T hzx,
                                             const T* __restrict__ ce, const T* __restrict__ cl, T* __restrict__ J,
                                             const T* __restrict__ cj, const T* __restrict__ sg, int use_cond,
                                             const Geom& g, const Metric<T>& mt, const BeamArgs& b,
                                             const PlaneArgs& pl, const StepArgs& st, long long n, int i0, int j,
                                             int k, const unsigned short* __restrict__ code = nullptr,
                                             const T* __restrict__ tab = nullptr) {
    static_assert(!(CODED && MODE == 2), "the explicit-J pass reads dense coefficients");
    T cur[3][VEC];
    epass_curl<T, VEC>(hx, hy, hz, hxy, hzy, hxz, hyz, hyx, hzx, cur, i0, j, k, g, mt);
    T ex[VEC], ey[VEC], ez[VEC], kx[VEC], ky[VEC], kz[VEC];
    [[maybe_unused]] unsigned cd[VEC];
    const int ni = (int)n, N32 = (int)g.N;  // 32-bit offsets, as in hpass_eval
    const T* Es = Esrc + ni;
    ld_v<T, VEC>(ex, Es);
    ld_v<T, VEC>(ey, Es + N32);
    ld_v<T, VEC>(ez, Es + N32 + N32);
    if constexpr (CODED) {
        ld_codes<VEC>(cd, code + ni);
        tab_get_v<T, VEC>(tab, cd, 1, kx, ky, kz);
    } else {
        const T* cen = ce + ni;
        ldg_v<T, VEC>(kx, cen);
        ldg_v<T, VEC>(ky, cen + N32);
        ldg_v<T, VEC>(kz, cen + N32 + N32);
    }
    if constexpr (MODE == 2) {
        const bool on_line = b.active && (j == b.iys) && (b.ixs >= i0) && (b.ixs < i0 + VEC);
        double jb = 0.0;
        if (on_line) {
            long long sn;
            double vt;
            resolve_step(st, sn, vt);
            jb = beam_current(b, k, vt);
        }
        T jx[VEC], jy[VEC], jz[VEC], ax[VEC], ay[VEC], az[VEC];
        ld_v<T, VEC>(jx, J + n);
        ld_v<T, VEC>(jy, J + g.N + n);
        ld_v<T, VEC>(jz, J + 2 * g.N + n);
        ldg_v<T, VEC>(ax, cj + n);
        ldg_v<T, VEC>(ay, cj + g.N + n);
        ldg_v<T, VEC>(az, cj + 2 * g.N + n);
        if (on_line) {
#pragma unroll
            for (int e = 0; e < VEC; ++e)
                if (i0 + e == b.ixs) jz[e] = (T)jb;
        }
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            ex[e] = rfma(-ax[e], jx[e], rfma(kx[e], cur[0][e], ex[e]));
            ey[e] = rfma(-ay[e], jy[e], rfma(ky[e], cur[1][e], ey[e]));
            ez[e] = rfma(-az[e], jz[e], rfma(kz[e], cur[2][e], ez[e]));
        }
        if (use_cond) {
            T sx[VEC], sy_[VEC], szz[VEC];
            ldg_v<T, VEC>(sx, sg + n);
            ldg_v<T, VEC>(sy_, sg + g.N + n);
            ldg_v<T, VEC>(szz, sg + 2 * g.N + n);
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                jx[e] = rmul(sx[e], ex[e]);
                jy[e] = rmul(sy_[e], ey[e]);
                jz[e] = rmul(szz[e], ez[e]);
            }
            st_v<T, VEC>(J + n, jx);
            st_v<T, VEC>(J + g.N + n, jy);
            st_v<T, VEC>(J + 2 * g.N + n, jz);
        } else if (on_line) {
            J[2 * g.N + n + (b.ixs - i0)] = (T)jb;
        }
    } else {
        T lx[VEC], ly[VEC], lz[VEC];
        if constexpr (MODE == 1 && CODED) {
            tab_get_v<T, VEC>(tab, cd, 2, lx, ly, lz);
        } else if constexpr (MODE == 1) {
            const T* cln = cl + ni;
            ldg_v<T, VEC>(lx, cln);
            ldg_v<T, VEC>(ly, cln + N32);
            ldg_v<T, VEC>(lz, cln + N32 + N32);
        } else {
            zero_v<T, VEC>(lx);
            zero_v<T, VEC>(ly);
            zero_v<T, VEC>(lz);
        }
        epass_update<T, VEC, MODE>(ex, ey, ez, kx, ky, kz, lx, ly, lz, cur, J, n, i0, j, k, use_cond, g, b, pl, st);
    }
    T* Ed = Edst + ni;
    st_v<T, VEC>(Ed, ex);
    st_v<T, VEC>(Ed + N32, ey);
    st_v<T, VEC>(Ed + N32 + N32, ez);
}


template <typename T, int VEC, int MODE, bool CODED = false>
__device__ __forceinline__ void epass_at(T* __restrict__ E, const T* __restrict__ H, const T* __restrict__ ce,
                                         const T* __restrict__ cl, T* __restrict__ J, const T* __restrict__ cj,
                                         const T* __restrict__ sg, int use_cond, const Geom& g, const Metric<T>& mt,
                                         const BeamArgs& b, const PlaneArgs& pl, const StepArgs& st, long long n,
                                         const unsigned short* __restrict__ code = nullptr,
                                         const T* __restrict__ tab = nullptr) {
    int i0, j, k;
    cell_of(n, g, i0, j, k);
    const int ni = (int)n, N32 = (int)g.N, sy = (int)g.sy, sz = (int)g.sz;  // 32-bit offsets
    const T* Hx = H + ni;
    const T* Hy = Hx + N32;
    const T* Hz = Hy + N32;
    T hx[VEC], hy[VEC], hz[VEC];
    ldg_v<T, VEC>(hx, Hx);
    ldg_v<T, VEC>(hy, Hy);
    ldg_v<T, VEC>(hz, Hz);
    const bool yv = (j > 0) || (k > 0);
    const bool zv = (k > 0);
    T hxy[VEC], hzy[VEC], hxz[VEC], hyz[VEC];
    if (yv) {
        ldg_v<T, VEC>(hxy, Hx - sy);
        ldg_v<T, VEC>(hzy, Hz - sy);
    } else {
        zero_v<T, VEC>(hxy);
        zero_v<T, VEC>(hzy);
    }
    if (zv) {
        ldg_v<T, VEC>(hxz, Hx - sz);
        ldg_v<T, VEC>(hyz, Hy - sz);
    } else {
        zero_v<T, VEC>(hxz);
        zero_v<T, VEC>(hyz);
    }
    T hyx = T(0), hzx = T(0);
    if (ni > 0) {
        hyx = __ldg(Hy - 1);
        hzx = __ldg(Hz - 1);
    }
    epass_finish<T, VEC, MODE, CODED>(E, E, hx, hy, hz, hxy, hzy, hxz, hyz, hyx, hzx, ce, cl, J, cj, sg, use_cond, g,
                                      mt, b, pl, st, n, i0, j, k, code, tab);
}

// ---------------------------------------------------------------- cell pairs (odd Nx)
// Grids with Nx odd have no 2-cell vectors inside rows, but when N is even the flat
// index splits into pairs (n, n+1), n even, that are 8-byte aligned in every component.
// A pair reads its own values as pairs and its neighbours at odd offsets one by one, and
// each of its two cells keeps its own (i, j, k): a pair may straddle two rows (the last
// cell of a row and the first of the next) or two planes, exactly the flat-index
// neighbours of the reference's curl, so no warp takes a separate path there.  Each cell
// gets the inputs the 1-wide kernels give it (hpass_at / epass_at with VEC = 1) and the
// same arithmetic (hpass_cells / epass_curl / epass_update), hence the same bits.
__device__ __forceinline__ void pair_cells(long long n, const Geom& g, int (&i)[2], int (&j)[2], int (&k)[2]) {
    cell_of(n, g, i[0], j[0], k[0]);
    i[1] = i[0] + 1;
    j[1] = j[0];
    k[1] = k[0];
    if (i[1] == g.nx) {
        i[1] = 0;
        if (++j[1] == g.ny) {
            j[1] = 0;
            ++k[1];
        }
    }
}

// the two values at p (8-byte aligned for FP32); RO: through the read-only path (inputs
// the kernel does not write)
template <typename T, bool RO>
__device__ __forceinline__ void ld_pair(T (&r)[2], const T* p) {
    if constexpr (sizeof(T) == 4) {
        const float2 t = RO ? __ldg(reinterpret_cast<const float2*>(p)) : *reinterpret_cast<const float2*>(p);
        r[0] = t.x;
        r[1] = t.y;
    } else {  // FP64: 16-byte aligned too (n and N even)
        const double2 t = RO ? __ldg(reinterpret_cast<const double2*>(p)) : *reinterpret_cast<const double2*>(p);
        r[0] = t.x;
        r[1] = t.y;
    }
}

// H pass of the cell pair at even flat index n (coded coefficients)
template <typename T>
__device__ __forceinline__ void hpass_pair_at(const T* __restrict__ E, T* __restrict__ H, const Geom& g,
                                              const Metric<T>& mt, long long n, const unsigned short* __restrict__ code,
                                              const T* __restrict__ tab) {
    int i[2], j[2], k[2];
    pair_cells(n, g, i, j, k);
    const T* Ex = E;
    const T* Ey = E + g.N;
    const T* Ez = E + 2 * g.N;
    T ex[2], ey[2], ez[2], hx[2], hy[2], hz[2];
    ld_pair<T, true>(ex, Ex + n);
    ld_pair<T, true>(ey, Ey + n);
    ld_pair<T, true>(ez, Ez + n);
    ld_pair<T, false>(hx, H + n);
    ld_pair<T, false>(hy, H + g.N + n);
    ld_pair<T, false>(hz, H + 2 * g.N + n);
    const unsigned cc = __ldg(reinterpret_cast<const unsigned*>(code + n));
    T eyn = T(0), ezn = T(0);  // past the pair: (n + 2)
    if (n + 2 < g.N) {
        eyn = __ldg(Ey + n + 2);
        ezn = __ldg(Ez + n + 2);
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const long long m = n + e;
        const bool yv = (j[e] + 1 < g.ny) || (k[e] + 1 < g.nz);
        const bool zv = k[e] + 1 < g.nz;
        T exy[1] = {yv ? __ldg(Ex + m + g.sy) : T(0)}, ezy[1] = {yv ? __ldg(Ez + m + g.sy) : T(0)};
        T exz[1] = {zv ? __ldg(Ex + m + g.sz) : T(0)}, eyz[1] = {zv ? __ldg(Ey + m + g.sz) : T(0)};
        T a[1] = {ex[e]}, b[1] = {ey[e]}, c[1] = {ez[e]};
        T px[1] = {hx[e]}, py[1] = {hy[e]}, pz[1] = {hz[e]};
        const unsigned cd[1] = {e ? (cc >> 16) : (cc & 0xffffu)};
        T cx[1], cy[1], cz[1];
        tab_get_v<T, 1>(tab, cd, 0, cx, cy, cz);
        hpass_cells<T, 1>(a, b, c, exy, ezy, exz, eyz, e ? eyn : ey[1], e ? ezn : ez[1], px, py, pz, cx, cy, cz, i[e],
                          j[e], k[e], g, mt);
        hx[e] = px[0];
        hy[e] = py[0];
        hz[e] = pz[0];
    }
    st_v<T, 2>(H + n, hx);
    st_v<T, 2>(H + g.N + n, hy);
    st_v<T, 2>(H + 2 * g.N + n, hz);
}

// E pass (MODE 0 or 1, coded coefficients) of the cell pair at even flat index n
template <typename T, int MODE>
__device__ __forceinline__ void epass_pair_at(T* __restrict__ E, const T* __restrict__ H, T* __restrict__ J,
                                              int use_cond, const Geom& g, const Metric<T>& mt, const BeamArgs& b,
                                              const StepArgs& st, long long n, const unsigned short* __restrict__ code,
                                              const T* __restrict__ tab, const PlaneArgs& pl = PlaneArgs{}) {
    int i[2], j[2], k[2];
    pair_cells(n, g, i, j, k);
    const T* Hx = H;
    const T* Hy = H + g.N;
    const T* Hz = H + 2 * g.N;
    T hx[2], hy[2], hz[2], ex[2], ey[2], ez[2];
    ld_pair<T, true>(hx, Hx + n);
    ld_pair<T, true>(hy, Hy + n);
    ld_pair<T, true>(hz, Hz + n);
    ld_pair<T, false>(ex, E + n);
    ld_pair<T, false>(ey, E + g.N + n);
    ld_pair<T, false>(ez, E + 2 * g.N + n);
    const unsigned cc = __ldg(reinterpret_cast<const unsigned*>(code + n));
    T hyp = T(0), hzp = T(0);  // before the pair: (n - 1)
    if (n > 0) {
        hyp = __ldg(Hy + n - 1);
        hzp = __ldg(Hz + n - 1);
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const long long m = n + e;
        const bool yv = (j[e] > 0) || (k[e] > 0);
        const bool zv = k[e] > 0;
        T hxy[1] = {yv ? __ldg(Hx + m - g.sy) : T(0)}, hzy[1] = {yv ? __ldg(Hz + m - g.sy) : T(0)};
        T hxz[1] = {zv ? __ldg(Hx + m - g.sz) : T(0)}, hyz[1] = {zv ? __ldg(Hy + m - g.sz) : T(0)};
        T a[1] = {hx[e]}, bb[1] = {hy[e]}, c[1] = {hz[e]};
        T cur[3][1];
        epass_curl<T, 1>(a, bb, c, hxy, hzy, hxz, hyz, e ? hy[0] : hyp, e ? hz[0] : hzp, cur, i[e], j[e], k[e], g, mt);
        const unsigned cd[1] = {e ? (cc >> 16) : (cc & 0xffffu)};
        T kx[1], ky[1], kz[1], lx[1], ly[1], lz[1];
        tab_get_v<T, 1>(tab, cd, 1, kx, ky, kz);
        if constexpr (MODE == 1) {
            tab_get_v<T, 1>(tab, cd, 2, lx, ly, lz);
        } else {
            lx[0] = ly[0] = lz[0] = T(0);
        }
        T fx[1] = {ex[e]}, fy[1] = {ey[e]}, fz[1] = {ez[e]};
        epass_update<T, 1, MODE>(fx, fy, fz, kx, ky, kz, lx, ly, lz, cur, J, m, i[e], j[e], k[e], use_cond, g, b, pl,
                                 st);
        ex[e] = fx[0];
        ey[e] = fy[0];
        ez[e] = fz[0];
    }
    st_v<T, 2>(E + n, ex);
    st_v<T, 2>(E + g.N + n, ey);
    st_v<T, 2>(E + 2 * g.N + n, ez);
}

template <typename T, int VEC, int MODE>
__global__ void __launch_bounds__(256, 3) k_epass(T* __restrict__ E, const T* __restrict__ H,
                                               const T* __restrict__ ce, const T* __restrict__ cl,
                                               T* __restrict__ J, const T* __restrict__ cj,
                                               const T* __restrict__ sg, int use_cond, Geom g,
                                               Metric<T> mt, BeamArgs b, PlaneArgs pl, StepArgs st) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.N / VEC) return;
    epass_at<T, VEC, MODE>(E, H, ce, cl, J, cj, sg, use_cond, g, mt, b, pl, st, v * VEC);
}

// the E pass (MODE 0 or 1) with coded coefficients (ce, cl from the code table)
template <typename T, int VEC, int MODE>
__global__ void __launch_bounds__(256, 3) k_epass_coded(T* __restrict__ E, const T* __restrict__ H,
                                                     T* __restrict__ J, int use_cond, Geom g, Metric<T> mt,
                                                     BeamArgs b, PlaneArgs pl, StepArgs st,
                                                     const unsigned short* __restrict__ code,
                                                     const T* __restrict__ tab, long long ahead) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.N / VEC) return;
    if (ahead > 0 && (v + ahead) * VEC < g.N) {  // as in k_hpass_coded
        const long long m = (v + ahead) * VEC;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            prefetch_l2(E + c * g.N + m);
            prefetch_l2(H + c * g.N + m);
        }
        prefetch_l2(code + m);
    }
    epass_at<T, VEC, MODE, true>(E, H, nullptr, nullptr, J, nullptr, nullptr, use_cond, g, mt, b, pl, st, v * VEC,
                                 code, tab);
}

// The coded two-pass passes on cell pairs (Nx odd, N even: grids with no 2-cell vectors
// inside rows).  ahead > 0: the thread first asks L2 for E, H and the codes of the pair
// `ahead` pairs on, the one a thread of the next resident wave of CTAs works on.
template <typename T>
__device__ __forceinline__ void pair_prefetch(const T* E, const T* H, const unsigned short* code, long long N,
                                              long long v, long long ahead) {
    if (ahead > 0 && (v + ahead) * 2 < N) {
        const long long m = (v + ahead) * 2;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            prefetch_l2(E + c * N + m);
            prefetch_l2(H + c * N + m);
        }
        prefetch_l2(code + m);
    }
}

template <typename T>
__global__ void __launch_bounds__(256, 4) k_hpass_pair(const T* __restrict__ E, T* __restrict__ H, Geom g,
                                                    Metric<T> mt, const unsigned short* __restrict__ code,
                                                    const T* __restrict__ tab, long long ahead) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.N / 2) return;
    pair_prefetch<T>(E, H, code, g.N, v, ahead);
    hpass_pair_at<T>(E, H, g, mt, v * 2, code, tab);
}

template <typename T, int MODE>
__global__ void __launch_bounds__(256, 4) k_epass_pair(T* __restrict__ E, const T* __restrict__ H,
                                                    T* __restrict__ J, int use_cond, Geom g, Metric<T> mt,
                                                    BeamArgs b, PlaneArgs pl, StepArgs st,
                                                    const unsigned short* __restrict__ code,
                                                    const T* __restrict__ tab, long long ahead) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.N / 2) return;
    pair_prefetch<T>(E, H, code, g.N, v, ahead);
    epass_pair_at<T, MODE>(E, H, J, use_cond, g, mt, b, st, v * 2, code, tab, pl);
}

// ---------------------------------------------------------------- fused step (2.5-D)
// One launch takes a whole leapfrog step and touches each value once: E^n and H^(n-1/2)
// are read from (Ein, Hin), E^(n+1) and H^(n+1/2) written to (Eout, Hout).  With
// separate input and output buffers every read of an old value is safe wherever the
// other CTAs are, so no CTA waits for another.  A CTA owns a tile of FX = 32*VEC cells
// along x and FY rows along y (one warp per row) plus one halo warp, and marches
// through a range of z planes.  For plane k
//   1. the row warps compute the new H of the tile (hpass_eval, the code of the
//      two-pass H kernel) and store it to Hout and to a shared plane buffer; the halo
//      warp computes, from the old fields, the new H of the row below the tile (flat
//      index n - Nx) and of the cell before each row segment (n - 1): the values the E
//      update needs from outside the tile.  Neighbours are flat-index neighbours, so the
//      row crossings of the reference's curl matrix are kept;
//   2. after one barrier the row warps update E of the tile from the shared planes k
//      and k-1 (epass_curl + epass_update, the code of the two-pass E kernel; the
//      coefficients ce, cl were loaded before the H update) and store it to Eout.
// Three plane buffers rotate: a buffer is rewritten two planes after its last read, so
// one barrier per plane suffices.  A CTA whose z range starts at k0 > 0 first computes
// the new H of plane k0-1 for its tile (not stored to Hout: the CTA below owns it).
// Per cell the step moves the fused algorithmic bytes (E, H read and written once; ch,
// ce and cl read once); halo reads of the neighbouring tiles hit L2.
// planes ahead whose first-touch data (E of plane k+PF+1 along x and y, E_z, H and the
// codes of plane k+PF) a row warp of the coded step asks L2 to fetch while it works on
// plane k; 0: off.  On the 512x512x1024 pillbox (4 rows) distances 0, 1, 2, 3 first ran
// 2.89, 2.62, 2.58 and 2.70 ms per step; with the explicitly rounded arithmetic and 32-bit
// offsets, 1, 2, 3 run 2.654, 2.677 and 2.706 ms (autotuned shapes).  The same prefetch
// for the halo row gained nothing.
#ifndef FIT_FUSED_PREFETCH
#define FIT_FUSED_PREFETCH 1
#endif


template <typename T, int VEC, int FY>
struct FusedShared {
    T h[3][3][FY + 1][32 * VEC];  // [plane buffer][component][row + 1 (row 0: below the tile)][x]
    T hx1[3][2][FY + 1];          // [plane buffer][Hy, Hz][row + 1]: the cell before each row segment
};

// The march of one tile column (bx, by) through planes k0 .. k1-1 (all threads of the
// CTA call it; the plane buffers in sm are free on entry).
template <typename T, int VEC, int FY, int MODE, bool CODED = false>
__device__ __forceinline__ void fused_march(const T* __restrict__ Ein, const T* __restrict__ Hin, T* __restrict__ Eout,
                                            T* __restrict__ Hout, const T* __restrict__ ch, const T* __restrict__ ce,
                                            const T* __restrict__ cl, T* __restrict__ J, int use_cond, const Geom& g,
                                            const Metric<T>& mt, const BeamArgs& b, const StepArgs& st, int bx, int by,
                                            int k0, int k1, FusedShared<T, VEC, FY>& sm,
                                            const unsigned short* __restrict__ code = nullptr,
                                            const T* __restrict__ tab = nullptr) {
    constexpr int FX = 32 * VEC;
    const int lane = threadIdx.x, ty = threadIdx.y;
    const bool halo = ty == FY;  // the halo warp
    const int i0 = bx * FX + lane * VEC;
    const int jt = by * FY;                   // first row of the tile
    const int j = halo ? jt : jt + ty;        // the halo warp works below row jt
    const bool on = i0 < g.nx && j < g.ny;
    const PlaneArgs pl{};
    const int xo = lane * VEC;
    if (k0 > 0 && on && !halo) {  // new H of plane k0-1 (the plane below the range) for the tile
        T hx[VEC], hy[VEC], hz[VEC];
        const long long n = (long long)i0 + g.sy * j + g.sz * (k0 - 1);
        hpass_eval<T, VEC, CODED>(Ein, Hin, ch, g, mt, n, i0, j, k0 - 1, hx, hy, hz, code, tab);
        const int bp = (k0 - 1) % 3;
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            sm.h[bp][0][ty + 1][xo + e] = hx[e];
            sm.h[bp][1][ty + 1][xo + e] = hy[e];
            sm.h[bp][2][ty + 1][xo + e] = hz[e];
        }
    }
    for (int k = k0; k < k1; ++k) {
        const int bc = k % 3, bp = (k + 2) % 3;
        const long long n = (long long)i0 + g.sy * j + g.sz * k;
        T hx[VEC], hy[VEC], hz[VEC];
        T kx[VEC], ky[VEC], kz[VEC], lx[VEC], ly[VEC], lz[VEC];
        unsigned cd[VEC];
        if constexpr (MODE != 1) {
            zero_v<T, VEC>(lx);
            zero_v<T, VEC>(ly);
            zero_v<T, VEC>(lz);
        }
        if (halo) {
            if (on) {  // the row below the tile: flat n - Nx (may wrap to plane k-1)
                T ax[VEC], ay[VEC], az[VEC];
                const long long m = n - g.sy;
                if (m >= 0) {
                    int mi, mj, mk;
                    cell_of(m, g, mi, mj, mk);
                    hpass_eval<T, VEC, CODED>(Ein, Hin, ch, g, mt, m, mi, mj, mk, ax, ay, az, code, tab);
                } else {
                    zero_v<T, VEC>(ax);
                    zero_v<T, VEC>(az);
                }
#pragma unroll
                for (int e = 0; e < VEC; ++e) {
                    sm.h[bc][0][0][xo + e] = ax[e];
                    sm.h[bc][2][0][xo + e] = az[e];
                }
            }
            // the cell before each row segment: flat n - 1 (may wrap)
            const int ib = bx * FX;
            if (lane < FY && ib < g.nx && jt + lane < g.ny) {
                const long long m = (long long)ib + g.sy * (jt + lane) + g.sz * k - 1;
                T ax[1], ay[1], az[1];
                if (m >= 0) {
                    int mi, mj, mk;
                    cell_of(m, g, mi, mj, mk);
                    hpass_eval<T, 1, CODED>(Ein, Hin, ch, g, mt, m, mi, mj, mk, ax, ay, az, code, tab);
                } else {
                    ay[0] = T(0);
                    az[0] = T(0);
                }
                sm.hx1[bc][0][lane + 1] = ay[0];
                sm.hx1[bc][1][lane + 1] = az[0];
            }
        } else if (on) {
            // the E update's coefficients do not depend on the new H: load them first so
            // their latency overlaps the H update and the barrier (coded: the codes; the
            // table entries are L1 hits, read after the barrier)
            const int ni = (int)n, N32 = (int)g.N, sz32 = (int)g.sz;  // 32-bit offsets, as in hpass_eval
            if constexpr (CODED && FIT_FUSED_PREFETCH > 0) {
                constexpr int PF = FIT_FUSED_PREFETCH;
                const T* Ep = Ein + ni;
                if (k + PF + 1 < g.nz) {
                    prefetch_l2(Ep + (PF + 1) * sz32);
                    prefetch_l2(Ep + N32 + (PF + 1) * sz32);
                }
                if (k + PF < g.nz) {
                    const int m = ni + PF * sz32;
                    const T* Hp = Hin + m;
                    prefetch_l2(Ein + m + N32 + N32);
                    prefetch_l2(Hp);
                    prefetch_l2(Hp + N32);
                    prefetch_l2(Hp + N32 + N32);
                    prefetch_l2(code + m);
                }
            }
            if constexpr (CODED) {
                ld_codes<VEC>(cd, code + ni);
            } else {
                const T* cen = ce + ni;
                ldg_v<T, VEC>(kx, cen);
                ldg_v<T, VEC>(ky, cen + N32);
                ldg_v<T, VEC>(kz, cen + N32 + N32);
                if constexpr (MODE == 1) {
                    const T* cln = cl + ni;
                    ldg_v<T, VEC>(lx, cln);
                    ldg_v<T, VEC>(ly, cln + N32);
                    ldg_v<T, VEC>(lz, cln + N32 + N32);
                }
            }
            hpass_eval<T, VEC, CODED>(Ein, Hin, ch, g, mt, n, i0, j, k, hx, hy, hz, code, tab, cd);
            T* Ho = Hout + ni;
            st_v<T, VEC>(Ho, hx);
            st_v<T, VEC>(Ho + N32, hy);
            st_v<T, VEC>(Ho + N32 + N32, hz);
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                sm.h[bc][0][ty + 1][xo + e] = hx[e];
                sm.h[bc][1][ty + 1][xo + e] = hy[e];
                sm.h[bc][2][ty + 1][xo + e] = hz[e];
            }
        }
        __syncthreads();
        if (on && !halo) {
            T hxy[VEC], hzy[VEC], hxz[VEC], hyz[VEC];
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                hxy[e] = sm.h[bc][0][ty][xo + e];
                hzy[e] = sm.h[bc][2][ty][xo + e];
            }
            if (k > 0) {
#pragma unroll
                for (int e = 0; e < VEC; ++e) {
                    hxz[e] = sm.h[bp][0][ty + 1][xo + e];
                    hyz[e] = sm.h[bp][1][ty + 1][xo + e];
                }
            } else {
                zero_v<T, VEC>(hxz);
                zero_v<T, VEC>(hyz);
            }
            const T hyx = lane > 0 ? sm.h[bc][1][ty + 1][xo - 1] : sm.hx1[bc][0][ty + 1];
            const T hzx = lane > 0 ? sm.h[bc][2][ty + 1][xo - 1] : sm.hx1[bc][1][ty + 1];
            T cur[3][VEC];
            epass_curl<T, VEC>(hx, hy, hz, hxy, hzy, hxz, hyz, hyx, hzx, cur, i0, j, k, g, mt);
            if constexpr (CODED) {
                tab_get_v<T, VEC>(tab, cd, 1, kx, ky, kz);
                if constexpr (MODE == 1) tab_get_v<T, VEC>(tab, cd, 2, lx, ly, lz);
            }
            T ex[VEC], ey[VEC], ez[VEC];
            const int ni = (int)n, N32 = (int)g.N;
            const T* Ei = Ein + ni;
            ldg_v<T, VEC>(ex, Ei);
            ldg_v<T, VEC>(ey, Ei + N32);
            ldg_v<T, VEC>(ez, Ei + N32 + N32);
            epass_update<T, VEC, MODE>(ex, ey, ez, kx, ky, kz, lx, ly, lz, cur, J, n, i0, j, k, use_cond, g, b, pl, st);
            T* Eo = Eout + ni;
            st_v<T, VEC>(Eo, ex);
            st_v<T, VEC>(Eo + N32, ey);
            st_v<T, VEC>(Eo + N32 + N32, ez);
        }
    }
}

// MB: CTAs per SM the register budget is sized for (the launch bound).  CODED: the
// coefficients come from code/tab instead of ch/ce/cl.
template <typename T, int VEC, int FY, int MB, int MODE, bool CODED>
__global__ void __launch_bounds__(32 * (FY + 1), MB)
    k_step_fused(const T* __restrict__ Ein, const T* __restrict__ Hin, T* __restrict__ Eout, T* __restrict__ Hout,
                 const T* __restrict__ ch, const T* __restrict__ ce, const T* __restrict__ cl, T* __restrict__ J,
                 int use_cond, Geom g, Metric<T> mt, BeamArgs b, StepArgs st, int zlen,
                 const unsigned short* __restrict__ code, const T* __restrict__ tab) {
    __shared__ FusedShared<T, VEC, FY> sm;
    const int k0 = blockIdx.z * zlen;
    fused_march<T, VEC, FY, MODE, CODED>(Ein, Hin, Eout, Hout, ch, ce, cl, J, use_cond, g, mt, b, st, blockIdx.x,
                                         blockIdx.y, k0, min(g.nz, k0 + zlen), sm, code, tab);
}

// ---------------------------------------------------------------- staged kernels
// Persistent kernels (one or two CTAs per SM) that walk the flat index space in chunks
// of CH cells.  For every chunk one elected thread issues bulk copies
// (cp.async.bulk global->shared, completion counted on an mbarrier) of each input
// stream -- the chunk's own cells plus the +-Nx row and +-Nx*Ny plane neighbours and
// a 16-byte pad for the +-1 neighbour -- into one of NST pipeline stages; the CTA
// computes from shared memory while the next NST-1 chunks are in flight.  DRAM
// latency is covered by the copies in flight, not by warp occupancy.  Requirements:
// Nx*sizeof(T) is a multiple of 16 bytes (all stream starts are then 16-byte aligned).
// Every wait is bounded (wlim polls): on expiry the kernel records FIT_ERR_TIMEOUT in
// *err, waits (bounded by kWaitLimit) for its own copies and returns.

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// bounded wait on phase `parity`; returns false when the bound expired
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, long long max_iter) {
    const unsigned a = smem_u32(bar);
    for (long long it = 0; it < max_iter; ++it) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// try_wait polls of a bounded wait (each waits up to ~a microsecond).  The waits for data
// take the context's limit (kWaitLimit unless fit_set_wait_limit changed it: a test of the
// give-up path sets 0); the drains after giving up always use kWaitLimit, so no copy lands
// in the shared memory of a CTA that has exited.
constexpr long long kWaitLimit = 1LL << 24;

struct Stream {
    int src;         // which input array (kernel specific)
    int comp;        // component block
    long long off;   // start relative to the chunk's first cell (elements)
    int pad;         // extra elements (the +-1 neighbour), multiple of the 16-byte width
};

// issue the copies of one chunk; returns the bytes expected on the barrier
template <typename T, int NS>
__device__ __forceinline__ unsigned issue_chunk(const T* const* srcs, const Stream (&ss)[NS], long long n0, int CH,
                                                long long N, T* stage, const int (&soff)[NS], unsigned long long* bar) {
    unsigned total = 0;
    long long beg[NS], end[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const long long a = n0 + ss[s].off;
        beg[s] = a < 0 ? 0 : a;
        long long e = a + CH + ss[s].pad;
        end[s] = e > N ? N : e;
        if (end[s] > beg[s]) total += (unsigned)((end[s] - beg[s]) * (long long)sizeof(T));
    }
    mbar_arrive_tx(bar, total);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (end[s] > beg[s]) {
            const long long a = n0 + ss[s].off;
            bulk_g2s(stage + soff[s] + (beg[s] - a), srcs[s] + (long long)ss[s].comp * N + beg[s],
                     (unsigned)((end[s] - beg[s]) * (long long)sizeof(T)), bar);
        }
    }
    return total;
}

template <typename T, int VEC>
__device__ __forceinline__ void lds_v(T (&r)[VEC], const T* p) {
    ld_v<T, VEC>(r, p);
}

// H pass streams: 0 Ex, 1 Ex+Nx, 2 Ex+NxNy, 3 Ey(+pad), 4 Ey+NxNy, 5 Ez(+pad), 6 Ez+Nx,
// 7-9 H, 10-12 ch
template <typename T, int VEC, int NST, int TPB>
__global__ void __launch_bounds__(TPB, 1) k_hpass_staged(const T* __restrict__ E, T* __restrict__ H,
                                                         const T* __restrict__ ch, Geom g, Metric<T> mt, int* err,
                                                         long long wlim) {
    constexpr int A = 16 / sizeof(T);
    constexpr int CH = TPB * VEC;
    constexpr int NS = 13;
    const Stream ss[NS] = {{0, 0, 0, 0},          {0, 0, g.sy, 0}, {0, 0, g.sz, 0}, {0, 1, 0, A}, {0, 1, g.sz, 0},
                           {0, 2, 0, A},          {0, 2, g.sy, 0}, {1, 0, 0, 0},    {1, 1, 0, 0}, {1, 2, 0, 0},
                           {2, 0, 0, 0},          {2, 1, 0, 0},    {2, 2, 0, 0}};
    int soff[NS];
    int stage_elems = 0;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        soff[s] = stage_elems;
        stage_elems += CH + ss[s].pad;
    }
    extern __shared__ __align__(128) unsigned char smem[];
    T* buf = reinterpret_cast<T*>(smem);
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + (size_t)NST * stage_elems * sizeof(T));
    const T* srcs[NS] = {E, E, E, E, E, E, E, H, H, H, ch, ch, ch};
    const long long nchunks = (g.N + CH - 1) / CH;
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) {
            const long long c = blockIdx.x + (long long)s * gridDim.x;
            if (c < nchunks) issue_chunk<T, NS>(srcs, ss, c * CH, CH, g.N, buf + (size_t)s * stage_elems, soff, &bars[s]);
        }
    }
    bool ok = true;
    long long it = 0;
    for (long long c = blockIdx.x; c < nchunks; c += gridDim.x, ++it) {
        const int s = (int)(it % NST);
        const unsigned parity = (unsigned)((it / NST) & 1);
        // every thread waits; the decision to give up is CTA-uniform
        if (!__syncthreads_and(mbar_wait(&bars[s], parity, wlim))) {
            ok = false;
            break;
        }
        const T* st = buf + (size_t)s * stage_elems;
        const long long n0 = c * CH;
        const long long n = n0 + (long long)tid * VEC;
        if (n < g.N) {
            int i0, j, k;
            cell_of(n, g, i0, j, k);
            const int o = tid * VEC;
            T ex[VEC], ey[VEC], ez[VEC], exy[VEC], ezy[VEC], exz[VEC], eyz[VEC];
            T hx[VEC], hy[VEC], hz[VEC], cx[VEC], cy[VEC], cz[VEC];
            lds_v<T, VEC>(ex, st + soff[0] + o);
            lds_v<T, VEC>(exy, st + soff[1] + o);
            lds_v<T, VEC>(exz, st + soff[2] + o);
            lds_v<T, VEC>(ey, st + soff[3] + o);
            lds_v<T, VEC>(eyz, st + soff[4] + o);
            lds_v<T, VEC>(ez, st + soff[5] + o);
            lds_v<T, VEC>(ezy, st + soff[6] + o);
            lds_v<T, VEC>(hx, st + soff[7] + o);
            lds_v<T, VEC>(hy, st + soff[8] + o);
            lds_v<T, VEC>(hz, st + soff[9] + o);
            lds_v<T, VEC>(cx, st + soff[10] + o);
            lds_v<T, VEC>(cy, st + soff[11] + o);
            lds_v<T, VEC>(cz, st + soff[12] + o);
            const T eyx = st[soff[3] + o + VEC];
            const T ezx = st[soff[5] + o + VEC];
            hpass_cells<T, VEC>(ex, ey, ez, exy, ezy, exz, eyz, eyx, ezx, hx, hy, hz, cx, cy, cz, i0, j, k, g, mt);
            st_v<T, VEC>(H + n, hx);
            st_v<T, VEC>(H + g.N + n, hy);
            st_v<T, VEC>(H + 2 * g.N + n, hz);
        }
        __syncthreads();  // every thread is done with stage s
        if (tid == 0) {
            const long long cn = c + (long long)NST * gridDim.x;
            if (cn < nchunks) {
                fence_proxy_async();
                issue_chunk<T, NS>(srcs, ss, cn * CH, CH, g.N, buf + (size_t)s * stage_elems, soff, &bars[s]);
            }
        }
    }
    if (!ok && tid == 0) {
        atomicExch(err, FIT_ERR_TIMEOUT);
        // drain: bounded waits on the stages of the chunks issued but not consumed
        for (long long q = it; q < it + NST; ++q)
            if (blockIdx.x + q * (long long)gridDim.x < nchunks)
                mbar_wait(&bars[q % NST], (unsigned)((q / NST) & 1), kWaitLimit);
    }
}

// E pass streams: 0 Hx, 1 Hx-Nx, 2 Hx-NxNy, 3 Hy(-pad), 4 Hy-NxNy, 5 Hz(-pad), 6 Hz-Nx,
// 7-9 E, 10-12 ce, 13-15 cl (MODE 1)
template <typename T, int VEC, int NST, int MODE, int TPB>
__global__ void __launch_bounds__(TPB, 1) k_epass_staged(T* __restrict__ E, const T* __restrict__ H,
                                                         const T* __restrict__ ce, const T* __restrict__ cl,
                                                         T* __restrict__ J, int use_cond, Geom g, Metric<T> mt,
                                                         BeamArgs b, PlaneArgs pl, StepArgs stp, int* err,
                                                         long long wlim) {
    constexpr int A = 16 / sizeof(T);
    constexpr int CH = TPB * VEC;
    constexpr int NS = MODE == 1 ? 16 : 13;
    Stream ss[NS];
    {
        const Stream base[16] = {{0, 0, 0, 0},      {0, 0, -g.sy, 0}, {0, 0, -g.sz, 0}, {0, 1, -A, A},
                                 {0, 1, -g.sz, 0},  {0, 2, -A, A},    {0, 2, -g.sy, 0}, {1, 0, 0, 0},
                                 {1, 1, 0, 0},      {1, 2, 0, 0},     {2, 0, 0, 0},     {2, 1, 0, 0},
                                 {2, 2, 0, 0},      {3, 0, 0, 0},     {3, 1, 0, 0},     {3, 2, 0, 0}};
#pragma unroll
        for (int s = 0; s < NS; ++s) ss[s] = base[s];
    }
    int soff[NS];
    int stage_elems = 0;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        soff[s] = stage_elems;
        stage_elems += CH + ss[s].pad;
    }
    extern __shared__ __align__(128) unsigned char smem[];
    T* buf = reinterpret_cast<T*>(smem);
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + (size_t)NST * stage_elems * sizeof(T));
    const T* srcs[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s)
        srcs[s] = s < 7 ? H : (s < 10 ? (const T*)E : (s < 13 ? ce : cl));
    const long long nchunks = (g.N + CH - 1) / CH;
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) {
            const long long c = blockIdx.x + (long long)s * gridDim.x;
            if (c < nchunks) issue_chunk<T, NS>(srcs, ss, c * CH, CH, g.N, buf + (size_t)s * stage_elems, soff, &bars[s]);
        }
    }
    bool ok = true;
    long long it = 0;
    for (long long c = blockIdx.x; c < nchunks; c += gridDim.x, ++it) {
        const int s = (int)(it % NST);
        const unsigned parity = (unsigned)((it / NST) & 1);
        // every thread waits; the decision to give up is CTA-uniform
        if (!__syncthreads_and(mbar_wait(&bars[s], parity, wlim))) {
            ok = false;
            break;
        }
        const T* st = buf + (size_t)s * stage_elems;
        const long long n0 = c * CH;
        const long long n = n0 + (long long)tid * VEC;
        if (n < g.N) {
            int i0, j, k;
            cell_of(n, g, i0, j, k);
            const int o = tid * VEC;
            T hx[VEC], hy[VEC], hz[VEC], hxy[VEC], hzy[VEC], hxz[VEC], hyz[VEC];
            lds_v<T, VEC>(hx, st + soff[0] + o);
            lds_v<T, VEC>(hxy, st + soff[1] + o);
            lds_v<T, VEC>(hxz, st + soff[2] + o);
            lds_v<T, VEC>(hy, st + soff[3] + A + o);
            lds_v<T, VEC>(hyz, st + soff[4] + o);
            lds_v<T, VEC>(hz, st + soff[5] + A + o);
            lds_v<T, VEC>(hzy, st + soff[6] + o);
            const T hyx = st[soff[3] + A + o - 1];
            const T hzx = st[soff[5] + A + o - 1];
            T cur[3][VEC];
            epass_curl<T, VEC>(hx, hy, hz, hxy, hzy, hxz, hyz, hyx, hzx, cur, i0, j, k, g, mt);
            T ex[VEC], ey[VEC], ez[VEC], kx[VEC], ky[VEC], kz[VEC], lx[VEC], ly[VEC], lz[VEC];
            lds_v<T, VEC>(ex, st + soff[7] + o);
            lds_v<T, VEC>(ey, st + soff[8] + o);
            lds_v<T, VEC>(ez, st + soff[9] + o);
            lds_v<T, VEC>(kx, st + soff[10] + o);
            lds_v<T, VEC>(ky, st + soff[11] + o);
            lds_v<T, VEC>(kz, st + soff[12] + o);
            if constexpr (MODE == 1) {
                lds_v<T, VEC>(lx, st + soff[13] + o);
                lds_v<T, VEC>(ly, st + soff[14] + o);
                lds_v<T, VEC>(lz, st + soff[15] + o);
            } else {
                zero_v<T, VEC>(lx);
                zero_v<T, VEC>(ly);
                zero_v<T, VEC>(lz);
            }
            epass_update<T, VEC, MODE>(ex, ey, ez, kx, ky, kz, lx, ly, lz, cur, J, n, i0, j, k, use_cond, g, b, pl,
                                       stp);
            st_v<T, VEC>(E + n, ex);
            st_v<T, VEC>(E + g.N + n, ey);
            st_v<T, VEC>(E + 2 * g.N + n, ez);
        }
        __syncthreads();
        if (tid == 0) {
            const long long cn = c + (long long)NST * gridDim.x;
            if (cn < nchunks) {
                fence_proxy_async();
                issue_chunk<T, NS>(srcs, ss, cn * CH, CH, g.N, buf + (size_t)s * stage_elems, soff, &bars[s]);
            }
        }
    }
    if (!ok && tid == 0) {
        atomicExch(err, FIT_ERR_TIMEOUT);
        // drain: bounded waits on the stages of the chunks issued but not consumed
        for (long long q = it; q < it + NST; ++q)
            if (blockIdx.x + q * (long long)gridDim.x < nchunks)
                mbar_wait(&bars[q % NST], (unsigned)((q / NST) & 1), kWaitLimit);
    }
}

// ---------------------------------------------------------------- coefficients
// FP64 build of ch, ce, cl (+ cj, sg for the explicit-J pass) from the material tensors.
// iA_c = 1/(L_p L_q) (wakis/gridFIT3D.py:277-280); itA_c = 1/(tL_p tL_q) or 0 where the
// dual area is 0 (wakis/gridFIT3D.py:298-304), then the periodic / ABC edits of
// wakis/boundaries.py:36-70,153-181 in the order they are applied: an edit along axis a
// sets itA_c(last index along a) = iA_c(index 0 along a) for c != a; the last edit wins.
struct CoeffArgs {
    const double* L[3];   // dx, dy, dz (FP64)
    const double* tL[3];  // UNEDITED dual lengths (FP64)
    int edits[6];         // axes in application order
    int n_edits;
    double dt;
    int use_cond;
};

__device__ __forceinline__ double coord_len(const double* const* L, int a, int i, int j, int k) {
    return a == 0 ? L[0][i] : (a == 1 ? L[1][j] : L[2][k]);
}

template <typename T>
__global__ void k_build_coeffs(const double* __restrict__ ieps, const double* __restrict__ imu,
                               const double* __restrict__ sigma, T* __restrict__ ch, T* __restrict__ ce,
                               T* __restrict__ cl, T* __restrict__ cj, T* __restrict__ sg, Geom g,
                               CoeffArgs a) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * g.N) return;
    const int c = (int)(idx / g.N);
    const long long n = idx - (long long)c * g.N;
    const int i = (int)(n % g.nx);
    const long long r = n / g.nx;
    const int j = (int)(r % g.ny);
    const int k = (int)(r / g.ny);
    const int p = (c + 1) % 3, q = (c + 2) % 3;  // the two other axes
    // primal inverse area
    const double iA = 1.0 / (coord_len(a.L, p, i, j, k) * coord_len(a.L, q, i, j, k));
    // dual inverse area with edits
    double itA;
    int edit_axis = -1;
    for (int e = a.n_edits - 1; e >= 0; --e) {
        const int ax = a.edits[e];
        if (ax == c) continue;
        const int last = ax == 0 ? g.nx - 1 : (ax == 1 ? g.ny - 1 : g.nz - 1);
        const int cur = ax == 0 ? i : (ax == 1 ? j : k);
        if (cur == last) {
            edit_axis = ax;
            break;
        }
    }
    if (edit_axis >= 0) {
        const int i2 = edit_axis == 0 ? 0 : i, j2 = edit_axis == 1 ? 0 : j, k2 = edit_axis == 2 ? 0 : k;
        itA = 1.0 / (coord_len(a.L, p, i2, j2, k2) * coord_len(a.L, q, i2, j2, k2));
    } else {
        const double ar = coord_len(a.tL, p, i, j, k) * coord_len(a.tL, q, i, j, k);
        itA = ar != 0.0 ? 1.0 / ar : 0.0;
    }
    const double pec = face_open(g.pec, c, i, j, k, g) ? 1.0 : 0.0;
    const double pmc = face_open(g.pmc, c, i, j, k, g) ? 1.0 : 0.0;
    const double ie = ieps[idx];
    ch[idx] = (T)(a.dt * (iA * imu[idx]) * pmc);
    ce[idx] = (T)(a.dt * (ie * itA) * pec);
    if (cl) cl[idx] = (T)(1.0 - a.dt * ie * sigma[idx]);
    if (cj) cj[idx] = (T)(a.dt * ie);
    if (sg) sg[idx] = (T)sigma[idx];
}

// ---------------------------------------------------------------- small kernels
// ---------------------------------------------------------------- coefficient code build
// Three passes over the dense coefficients of a context: (1) insert every cell's
// (ch, ce, cl) triple, keyed by a 64-bit hash of its bits, into an open-addressing table
// (one insert per distinct key and warp, others find their key already present);
// (2) number the occupied slots in slot order and copy their triples into the code
// table; (3) give every cell the code of its key and compare its triple with the code
// table bit for bit.  Any mismatch (a hash collision), a full table or more than
// kMaxCodes distinct triples leaves the context dense.  No pass waits on another thread.
constexpr int kCodeSlots = 1 << 17;
constexpr int kMaxCodes = 65535;
constexpr int kCodeProbes = 4096;  // probe bound; the table is at most half full while codes fit

template <typename T>
__device__ __forceinline__ unsigned long long word_bits(T v) {
    if constexpr (sizeof(T) == 4) return (unsigned long long)__float_as_uint(v);
    else return (unsigned long long)__double_as_longlong(v);
}

template <typename T>
__device__ __forceinline__ void coef_triple(const T* __restrict__ ch, const T* __restrict__ ce,
                                            const T* __restrict__ cl, long long N, long long n, T (&v)[9]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = ch[c * N + n];
        v[3 + c] = ce[c * N + n];
        v[6 + c] = cl ? cl[c * N + n] : T(0);
    }
}

// FNV-1a over the nine words, then the 64-bit finaliser of MurmurHash3; 0 marks an
// empty slot and is never returned
template <typename T>
__device__ __forceinline__ unsigned long long triple_hash(const T (&v)[9]) {
    unsigned long long h = 0xcbf29ce484222325ULL;
#pragma unroll
    for (int i = 0; i < 9; ++i) h = (h ^ word_bits(v[i])) * 0x100000001b3ULL;
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdULL;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ULL;
    h ^= h >> 33;
    return h ? h : 1ULL;
}

// status: [0] too many triples (more than kMaxCodes inserted, or a probe bound hit),
// [1] number of codes, [2] cells whose triple differs from its code's, [3] keys inserted
template <typename T>
__global__ void k_code_insert(const T* __restrict__ ch, const T* __restrict__ ce, const T* __restrict__ cl,
                              long long N, unsigned long long* keys, T* __restrict__ vals, int* status) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    // the trip count and the stop decision are uniform across each warp, so the
    // warp-wide match below is legal
    for (long long base = (long long)blockIdx.x * blockDim.x; base < N; base += stride) {
        int stop = 0;
        if ((threadIdx.x & 31) == 0) stop = *(volatile int*)&status[0];
        if (__shfl_sync(0xffffffffu, stop, 0)) break;
        const long long n = base + threadIdx.x;
        const bool valid = n < N;
        T v[9];
        unsigned long long h = 0;
        if (valid) {
            coef_triple<T>(ch, ce, cl, N, n, v);
            h = triple_hash<T>(v);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, h);
        if (!valid || (int)(__ffs(peers) - 1) != (int)(threadIdx.x & 31)) continue;
        unsigned slot = (unsigned)h & (kCodeSlots - 1);
        int p = 0;
        for (; p < kCodeProbes; ++p) {
            const unsigned long long cur = keys[slot];
            if (cur == h) break;
            if (cur == 0) {
                const unsigned long long old = atomicCAS(&keys[slot], 0ULL, h);
                if (old == 0) {
#pragma unroll
                    for (int i = 0; i < 9; ++i) vals[(long long)slot * 9 + i] = v[i];
                    if (atomicAdd(&status[3], 1) >= kMaxCodes) atomicExch(&status[0], 1);
                    break;
                }
                if (old == h) break;
            }
            slot = (slot + 1) & (kCodeSlots - 1);
        }
        if (p == kCodeProbes) atomicExch(&status[0], 1);
    }
}

// one block of 1024 threads, kCodeSlots / 1024 slots each
template <typename T>
__global__ void k_code_number(const unsigned long long* __restrict__ keys, const T* __restrict__ vals,
                              int* __restrict__ slot_code, T* __restrict__ tab, int* status) {
    __shared__ int part[1024];
    constexpr int per = kCodeSlots / 1024;
    const int a = threadIdx.x * per;
    int cnt = 0;
    for (int q = a; q < a + per; ++q) cnt += keys[q] != 0;
    part[threadIdx.x] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < 1024; ++t) {
            const int c = part[t];
            part[t] = run;
            run += c;
        }
        status[1] = run;
    }
    __syncthreads();
    int code = part[threadIdx.x];
    for (int q = a; q < a + per; ++q) {
        if (keys[q] == 0) {
            slot_code[q] = -1;
            continue;
        }
        slot_code[q] = code;
        if (code < kMaxCodes) {
            for (int grp = 0; grp < 3; ++grp) {
                for (int c = 0; c < 3; ++c) tab[(long long)code * 12 + grp * 4 + c] = vals[(long long)q * 9 + grp * 3 + c];
                tab[(long long)code * 12 + grp * 4 + 3] = T(0);
            }
        }
        ++code;
    }
}

template <typename T>
__global__ void k_code_assign(const T* __restrict__ ch, const T* __restrict__ ce, const T* __restrict__ cl,
                              long long N, const unsigned long long* __restrict__ keys,
                              const int* __restrict__ slot_code, const T* __restrict__ tab,
                              unsigned short* __restrict__ code, int* status) {
    if (status[0]) return;  // too many triples: the context stays dense
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += stride) {
        T v[9];
        coef_triple<T>(ch, ce, cl, N, n, v);
        const unsigned long long h = triple_hash<T>(v);
        unsigned slot = (unsigned)h & (kCodeSlots - 1);
        int c = -1;
        for (int p = 0; p < kCodeProbes; ++p) {
            const unsigned long long cur = keys[slot];
            if (cur == h) {
                c = slot_code[slot];
                break;
            }
            if (cur == 0) break;
            slot = (slot + 1) & (kCodeSlots - 1);
        }
        bool same = c >= 0 && c < kMaxCodes;
        if (same) {
            code[n] = (unsigned short)c;
            for (int grp = 0; grp < 3; ++grp)
                for (int q = 0; q < 3; ++q)
                    same = same && word_bits(tab[(long long)c * 12 + grp * 4 + q]) == word_bits(v[grp * 3 + q]);
        }
        if (!same) atomicAdd(&status[2], 1);
    }
}

template <typename T>
__global__ void k_zero_ghosts(T* __restrict__ E, T* __restrict__ H, Geom g) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const int i = (int)(n % g.nx);
    const long long r = n / g.nx;
    const int j = (int)(r % g.ny);
    const int k = (int)(r / g.ny);
    const bool xl = i == g.nx - 1, yl = j == g.ny - 1, zl = k == g.nz - 1;
    if (yl || zl) H[n] = T(0);
    if (xl || zl) H[g.N + n] = T(0);
    if (xl || yl) H[2 * g.N + n] = T(0);
    if (xl) E[n] = T(0);
    if (yl) E[g.N + n] = T(0);
    if (zl) E[2 * g.N + n] = T(0);
}

// copy the index-1 plane to the index-0 plane along `axis`, all components of E and H
template <typename T>
__global__ void k_abc_lo(T* __restrict__ E, T* __restrict__ H, Geom g, int axis) {
    const int pa = axis == 0 ? g.ny : g.nx;
    const int pb = axis == 2 ? g.ny : g.nz;
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= 6LL * pa * pb) return;
    const int f = (int)(m / ((long long)pa * pb));
    const long long q = m - (long long)f * pa * pb;
    const int u = (int)(q % pa), w = (int)(q / pa);
    int i, j, k;
    long long s;
    if (axis == 0) { i = 0; j = u; k = w; s = 1; }
    else if (axis == 1) { i = u; j = 0; k = w; s = g.sy; }
    else { i = u; j = w; k = 0; s = g.sz; }
    T* F = (f < 3 ? E : H) + (long long)(f % 3) * g.N;
    const long long n = i + g.sy * j + g.sz * k;
    F[n] = F[n + s];
}

// hard plane source + wake taps + step counter (one launch per step, before the H pass)
struct TapArgs {
    int nlines;
    const long long* base;  // flat index of E_z(lx, ly, kskip) per line
    int ns;
    long long nsteps;
    const long long* row_ptr;
    const int* ent_m;
    const int* ent_k0;
    const int* ent_cnt;
    const double* dz;
    double* acc;   // nlines*ns running sums
    double* comp;  // nlines*ns Neumaier compensation
};

__device__ __forceinline__ void neumaier_add(double& s, double& c, double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// wake taps of E^n: the (s, z) pairs whose time index is step n add Ez*dz to their
// line's running sum (FP64, compensated).  Called by all threads of one block.  The
// entries of a step are ordered by s index; the runs of one s index (one accumulator
// per line) are summed by one thread, the one holding the first of them.
template <typename T>
__device__ __forceinline__ void wake_taps(const T* __restrict__ E, const Geom& g, const TapArgs& tp, long long n,
                                          int slice = 0, int slices = 1) {
    if (tp.nlines > 0 && n >= 0 && n < tp.nsteps) {
        const long long r0 = tp.row_ptr[n], r1 = tp.row_ptr[n + 1];
        const long long cnt = (r1 - r0) * tp.nlines;
        const T* Ez = E + 2 * g.N;
        // work items t: this block's slice of them, blockDim.x apart
        for (long long t = threadIdx.x + (long long)slice * blockDim.x; t < cnt; t += (long long)blockDim.x * slices) {
            const long long e = r0 + t / tp.nlines;
            const int l = (int)(t % tp.nlines);
            const int m = tp.ent_m[e];
            if (e > r0 && tp.ent_m[e - 1] == m) continue;  // summed with the group's first run
            double s = tp.acc[(long long)l * tp.ns + m], cc = tp.comp[(long long)l * tp.ns + m];
            for (long long f = e; f < r1 && tp.ent_m[f] == m; ++f) {
                const int k0 = tp.ent_k0[f], c = tp.ent_cnt[f];
                for (int q = 0; q < c; ++q) {
                    const double ez = (double)Ez[tp.base[l] + g.sz * (long long)(k0 + q)];
                    neumaier_add(s, cc, __dmul_rn(ez, tp.dz[k0 + q]));
                }
            }
            tp.acc[(long long)l * tp.ns + m] = s;
            tp.comp[(long long)l * tp.ns + m] = cc;
        }
    }
}

// Ez line history (the reference's Ez.h5 dump, wakis/routines.py:438-446): E_z of each
// recorded line over all z, taken with the wake taps (after the source update, before
// the step), stored hist[n - n0][line][k] in the field dtype.
struct RecordArgs {
    void* hist;
    int nlines;
    long long base[9];  // flat index of E_z(lx, ly, 0) per line
    long long n0, nsteps;
};

// J_z line history (the reference's Jz.h5 dump of wakesolve(save_J=True),
// wakis/routines.py:440-445): J_z on the recorded lines after the beam update and before
// the step.  J is sigma*E of the previous step there (the reference's J = sigma*E, a
// float64 product stored in the field dtype), and the beam current on the beam line.
struct JRecordArgs {
    void* hist;  // [step][line][k] in the field dtype
    int nlines;
    int pad;
    long long base[9];  // flat index of J_z(lx, ly, 0) per line
    long long n0, nsteps;
    const double* sig;  // sigma_z on the lines, [line][k] (device)
    BeamArgs beam;
    const double* vt_table;  // device loops: v*t of step n
    long long vt_len;
    double vt_host;  // host-driven steps: v*t of this step
};

template <typename T>
__global__ void k_prologue(T* __restrict__ E, T* __restrict__ H, Geom g, PlaneArgs pl, TapArgs tp,
                           long long n_arg, long long* d_step, RecordArgs rec, JRecordArgs jr) {
    const long long n = d_step ? *d_step : n_arg;
    // plane source
    if (pl.active && n >= 0 && n < pl.len) {
        const int w = pl.x1 - pl.x0, h = pl.y1 - pl.y0;
        const double c1 = pl.c1[n], c2 = pl.c2[n], gt = pl.gt[n];
        for (int t = threadIdx.x; t < w * h; t += blockDim.x) {
            const int i = pl.x0 + t % w, j = pl.y0 + t / w;
            const double pv = pl.prof ? pl.prof[t] : 1.0;
            const long long c = i + g.sy * j + g.sz * pl.zs;
            if (pl.stash) pl.stash[t] = (double)E[c];
            H[g.N + c] = (T)__dmul_rn(__dmul_rn(c1, pv), gt);
            E[c] = (T)__dmul_rn(__dmul_rn(c2, pv), gt);
        }
    }
    if (rec.nlines > 0 && n >= rec.n0 && n < rec.n0 + rec.nsteps) {
        T* h = static_cast<T*>(rec.hist) + (n - rec.n0) * rec.nlines * (long long)g.nz;
        const T* Ez = E + 2 * g.N;
        for (int t = threadIdx.x; t < rec.nlines * g.nz; t += blockDim.x) {
            const int l = t / g.nz, k = t - l * g.nz;
            h[t] = Ez[rec.base[l] + g.sz * k];
        }
    }
    if (jr.nlines > 0 && n >= jr.n0 && n < jr.n0 + jr.nsteps) {
        T* h = static_cast<T*>(jr.hist) + (n - jr.n0) * jr.nlines * (long long)g.nz;
        const T* Ez = E + 2 * g.N;
        const double vt = d_step ? ((jr.vt_table && n < jr.vt_len) ? jr.vt_table[n] : 0.0) : jr.vt_host;
        for (int t = threadIdx.x; t < jr.nlines * g.nz; t += blockDim.x) {
            const int l = t / g.nz, k = t - l * g.nz;
            if (jr.beam.active && jr.base[l] == jr.beam.ixs + g.sy * jr.beam.iys)
                h[t] = (T)beam_current(jr.beam, k, vt);
            else
                h[t] = (T)__dmul_rn(jr.sig[t], (double)Ez[jr.base[l] + g.sz * k]);
        }
    }
    wake_taps<T>(E, g, tp, n);
    if (d_step) {
        __syncthreads();
        if (threadIdx.x == 0) *d_step = n + 1;
    }
}

// Field monitor (FieldMonitor.update, wakis/field_monitors.py:59-101): running DFT of E
// at nf frequencies, acc[f][c][n] += E_c[n] * phase[f], accumulated in FP64 (complex128),
// with the operation order of the reference's complex product of a real field value by
// the phase: re += e*pr, im += e*pi (no fused multiply-add).  With single set the
// products are rounded to FP32 first: numpy evaluates an FP32 field times a phase taken
// from an FP32 time in complex64.  The phase row of a device-loop step is
// phases[(*d_step - 1) - n0] (the prologue advanced the counter before the passes).
struct MonitorArgs {
    int nf;
    int single;             // products in FP32 (FP32 field, complex64 phases)
    const double2* phases;  // steps x nf, or the nf phases of one host-driven update
    long long n0, nsteps;   // device loop: steps n0 <= n < n0 + nsteps are monitored
    double2* acc;           // [3][nf][N]
};

template <typename T>
__global__ void k_monitor(const T* __restrict__ E, long long N, MonitorArgs m, const long long* d_step, long long n_arg) {
    const double2* ph = m.phases;
    if (d_step || n_arg >= 0) {
        const long long n = d_step ? *d_step - 1 : n_arg;
        if (n < m.n0 || n >= m.n0 + m.nsteps) return;
        ph += (n - m.n0) * m.nf;
    }
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < 3 * N;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long c = idx / N, n = idx - c * N;
        const T ev = E[idx];
        const double e = (double)ev;
        for (int f = 0; f < m.nf; ++f) {
            const double2 p = ph[f];
            double2* a = m.acc + (c * m.nf + f) * N + n;
            double2 v = *a;
            double px, py;
            if (sizeof(T) == 4 && m.single) {
                px = (double)__fmul_rn((float)ev, (float)p.x);
                py = (double)__fmul_rn((float)ev, (float)p.y);
            } else {
                px = __dmul_rn(e, p.x);
                py = __dmul_rn(e, p.y);
            }
            v.x = __dadd_rn(v.x, px);
            v.y = __dadd_rn(v.y, py);
            *a = v;
        }
    }
}

// J = sigma*E (field dtype) and the beam line
template <typename T>
__global__ void k_materialize_J(const T* __restrict__ E, T* __restrict__ J, const double* __restrict__ sigma,
                                Geom g, int use_cond) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * g.N) return;
    if (use_cond) J[idx] = (T)sigma[idx] * E[idx];
}
template <typename T>
__global__ void k_beam_line(T* __restrict__ J, Geom g, BeamArgs b, double vt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.nz) return;
    J[2 * g.N + b.ixs + g.sy * b.iys + g.sz * k] = (T)beam_current(b, k, vt);
}

// wake post-processing: combine lines with the non-reset accumulator of the reference,
// then exclusive prefix sums (x ds) and the Panofsky-Wenzel central differences.
// One block of 1024 threads.  acc == nullptr: wp3d already holds the combined lines.
// The lines form a side x side square (row-major, side = 2n+1, n >= 1); the transverse
// wake reads lines (n+1, n), (n-1, n), (n, n+1), (n, n-1); side 0: longitudinal only.
__global__ void k_wake_finalize(const double* __restrict__ acc, const double* __restrict__ comp, int nlines,
                                int ns, double qscale, double ds, double dxf, double dyf,
                                double* __restrict__ wp3d, double* __restrict__ wpx, double* __restrict__ wpy,
                                double* __restrict__ scratch /* 4*ns */, int side) {
    // 1. line combination, sequential over lines, parallel over s
    for (int m = threadIdx.x; acc && m < ns; m += blockDim.x) {
        double prev = 0.0;
        for (int l = 0; l < nlines; ++l) {
            const double raw = acc[(long long)l * ns + m] + comp[(long long)l * ns + m];
            prev = (prev + raw) / qscale;
            wp3d[(long long)l * ns + m] = prev;
        }
    }
    __syncthreads();
    if (side < 3 || nlines != side * side) return;
    // 2. exclusive prefix sums of lines (n+1,n), (n-1,n), (n,n+1), (n,n-1) (row-major;
    // 7, 1, 5, 3 of the 3x3 square)
    __shared__ double part[1024];
    const int c0 = side / 2;
    const int lines[4] = {(c0 + 1) * side + c0, (c0 - 1) * side + c0, c0 * side + c0 + 1, c0 * side + c0 - 1};
    const int T = blockDim.x;
    const int chunk = (ns + T - 1) / T;
    for (int q = 0; q < 4; ++q) {
        const double* w = wp3d + (long long)lines[q] * ns;
        const int a = threadIdx.x * chunk, bnd = min(ns, a + chunk);
        double s = 0.0, c = 0.0;
        for (int m = a; m < bnd; ++m) neumaier_add(s, c, w[m]);
        part[threadIdx.x] = s + c;
        __syncthreads();
        if (threadIdx.x == 0) {
            double run = 0.0, rc = 0.0;
            for (int t = 0; t < T; ++t) {
                const double v = part[t];
                part[t] = run + rc;
                neumaier_add(run, rc, v);
            }
        }
        __syncthreads();
        s = part[threadIdx.x];
        c = 0.0;
        for (int m = a; m < bnd; ++m) {
            scratch[(long long)q * ns + m] = (s + c) * ds;  // sum of w[0:m]
            neumaier_add(s, c, w[m]);
        }
        __syncthreads();
    }
    for (int m = threadIdx.x; m < ns; m += blockDim.x) {
        wpx[m] = -(scratch[m] - scratch[ns + m]) / dxf;
        wpy[m] = -(scratch[2LL * ns + m] - scratch[3LL * ns + m]) / dyf;
    }
}

// Wake integral from a recorded Ez line history, the post-processing of an Ez file
// (wakis/wakeSolver.py:311-421 longitudinal, 423-551 over the 3x3 lines).  One thread
// per s index m.  The reference's operation order is kept exactly: lines in order, k
// ascending, plain FP64 sums of the rounded products Ez*dz (no FMA) continued from the
// previous line's result (the accumulator is not reset), divided by q*1e12 after each
// line.  ezt: [nlines][nz][nt], the reference's Ezt (nz, nt) per line; it: [nz][ns],
// the time index of tap (m, k) or -1 where the reference skips it (it >= nt); entries
// outside [0, nt) are skipped.
__global__ void k_wake_history(const double* __restrict__ ezt, int nlines, long long nt, int nz,
                               const int* __restrict__ it, int ns, const double* __restrict__ dz, double qscale,
                               double* __restrict__ wp3d) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= ns) return;
    double wp = 0.0;
    for (int l = 0; l < nlines; ++l) {
        const double* e = ezt + (long long)l * nz * nt;
        for (int k = 0; k < nz; ++k) {
            const int t = it[(long long)k * ns + m];
            if (t >= 0 && t < nt) wp = __dadd_rn(wp, __dmul_rn(e[(long long)k * nt + t], dz[k]));
        }
        wp = __ddiv_rn(wp, qscale);
        wp3d[(long long)l * ns + m] = wp;
    }
}

// FP64 direct DFT: stage 1 writes compensated partial sums of a slice of the time axis
// to scratch; stage 2 adds the slices.  Twiddle phase from the exact integer (b*t) mod n.
// The signal index is blockIdx.y: at most 65535 signals per launch.
constexpr int kDftMaxSignals = 65535;
__global__ void k_dft_partial(const double* __restrict__ x, int nsig, long long len, long long n, long long b0,
                              int nb, int nsplit, double2* __restrict__ part) {
    const int b = blockIdx.x;          // bin offset
    const int sgl = blockIdx.y;        // signal
    const int sp = blockIdx.z;         // slice
    const long long per = (len + nsplit - 1) / nsplit;
    const long long t0 = (long long)sp * per, t1 = min(len, t0 + per);
    const long long bin = b0 + b;
    double sr = 0.0, cr = 0.0, si = 0.0, ci = 0.0;
    const double* xs = x + (long long)sgl * len;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        const long long rr = (long long)(((unsigned long long)bin * (unsigned long long)t) % (unsigned long long)n);
        double sn, cs;
        sincospi(2.0 * (double)rr / (double)n, &sn, &cs);
        const double v = xs[t];
        neumaier_add(sr, cr, v * cs);
        neumaier_add(si, ci, -v * sn);
    }
    __shared__ double red_r[256], red_i[256];
    red_r[threadIdx.x] = sr + cr;
    red_i[threadIdx.x] = si + ci;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red_r[threadIdx.x] += red_r[threadIdx.x + w];
            red_i[threadIdx.x] += red_i[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[((long long)sgl * nsplit + sp) * nb + b] = make_double2(red_r[0], red_i[0]);
}

__global__ void k_dft_reduce(const double2* __restrict__ part, int nsig, int nb, int nsplit, double2* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nsig * nb) return;
    const int sgl = (int)(idx / nb), b = (int)(idx % nb);
    double sr = 0.0, cr = 0.0, si = 0.0, ci = 0.0;
    for (int sp = 0; sp < nsplit; ++sp) {
        const double2 v = part[((long long)sgl * nsplit + sp) * nb + b];
        neumaier_add(sr, cr, v.x);
        neumaier_add(si, ci, v.y);
    }
    out[idx] = make_double2(sr + cr, si + ci);
}

// ---------------------------------------------------------------- batched (pool) kernels
// Independent grids ("instances") advance together: one launch of a pass covers the
// cells of every instance of one vector-width class in a device work table.  Rows are
// ordered by class (4, 2, then 1 cells per vector: the widest that divides Nx) and each
// instance's flat index space is cut into tiles of kPoolTpb vectors, laid end to end;
// cls_t0 gives each class's tile range.  A persistent grid walks its class's tiles in
// grid-stride order; a CTA reads the descriptor of the instance it is in into shared
// memory and fetches the next one only when its tiles cross into another instance, so
// most tiles run without a barrier.  The grid does not depend
// on the table, so a captured graph serves every mix with the same classes present, and
// the table can change between graph replays.  Each instance keeps its own device step
// counter; an instance whose counter has reached its end is skipped, so instances that
// finish inside a chunk of steps cost one descriptor fetch per CTA from then on.  The
// per-cell arithmetic is hpass_at / epass_at, the code of the single-grid kernels, so a
// pooled instance gives bit-identical fields to the same grid run alone.
constexpr int kPoolMaxInst = 64;
constexpr int kPoolTpb = 256;
// classes: 0, 1, 2 = two-pass kernels with 4-, 2-, 1-wide vectors; 3, 4, 5 = the fused
// step on plane segments with 4-, 2-, 1-wide vectors (coded contexts with the fused step
// enabled and Nx <= kSegMaxNx)
constexpr int kPoolClasses = 6;
constexpr int kSegTpb = 256;    // threads of a fused CTA
constexpr int kSegWin = 1024;   // cells of the H window per plane: a segment and the Nx cells before it
constexpr int kSegMaxNx = 256;  // the fused class holds grids with Nx up to this (segments of >= 768 cells)

__host__ __device__ constexpr int pool_class(int vec) { return vec == 4 ? 0 : (vec == 2 ? 1 : 2); }
__host__ __device__ constexpr int pool_fused_class(int vec) { return vec == 4 ? 3 : (vec == 2 ? 4 : 5); }

template <typename T>
struct PoolInst {
    Geom g;
    Metric<T> mt;
    T* E;
    T* H;
    const T* ch;
    const T* ce;
    const T* cl;
    T* J;
    BeamArgs beam;
    TapArgs tap;
    long long* d_step;  // the instance's step counter, left at the next step by k_prologue_pool
    long long n0c;      // the step the instance takes at the chunk's first step
    const double* vt_table;
    long long vt_len;
    long long n_end;  // steps n < n_end are taken
    long long tile0;  // first tile (fused: work item) of the instance in its class
    long long ntile;  // tiles: ceil(nvec / kPoolTpb); fused: nseg * z ranges
    long long nvec;   // N / vec
    T* E2;            // fused: the second field buffers (steps alternate E,H <-> E2,H2)
    T* H2;
    int vec;          // cells per vector: 4, 2 or 1 (Nx % vec == 0)
    int mode;         // 0: lossless, 1: J = sigma*E folded into the loss factor
    int use_cond;
    int fused;        // 1: stepped by k_step_seg_pool
    int zlen;         // fused: planes per work item
    int pair;         // 1-wide class: 1 when N is even, stepped in cell pairs (nvec = N / 2)
    long long nseg;   // fused: plane segments, ceil(Nx*Ny / (kSegWin - Nx))
    const unsigned short* code;  // coded coefficients (nullptr: dense; two-pass classes only)
    const T* tab;
};

template <typename T>
struct PoolTable {
    int ninst;
    int pad;
    long long cls_t0[kPoolClasses + 1];  // tiles (work items) of class c: [cls_t0[c], cls_t0[c+1])
    PoolInst<T> inst[kPoolMaxInst];
};

// descriptor of the instance owning tile t into shared memory, and its current step
template <typename T>
__device__ __forceinline__ void pool_fetch(const PoolTable<T>* __restrict__ tab, int ninst, long long t,
                                           PoolInst<T>* si, long long* step, int s, double* vt) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tab->inst[mid].tile0 <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    static_assert(sizeof(PoolInst<T>) % 8 == 0, "descriptor copied in 8-byte words");
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&tab->inst[lo]);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(si);
    for (int w = threadIdx.x; w < (int)(sizeof(PoolInst<T>) / 8); w += blockDim.x) dst[w] = src[w];
    if (threadIdx.x == 0) {  // step s of the chunk and the beam's v*t at it
        const PoolInst<T>& d = tab->inst[lo];
        const long long n = d.n0c + s;
        *step = n;
        *vt = (d.vt_table && n >= 0 && n < d.vt_len) ? d.vt_table[n] : 0.0;
    }
}

// Walks the class's tiles in grid-stride order, so the CTAs in flight sweep the flat
// index space together and the +-row / +-plane neighbours of a tile are still in L2
// from the tiles before it (as in the single-grid kernels); body(si, v) runs vector v
// (instance-relative) of the instance in si, for the instances whose run has not ended.
// The descriptor is fetched again only when the tile leaves the cached instance: the
// test is uniform over the CTA, so the barriers around the fetch are too.
template <typename T, int VEC, typename Body>
__device__ __forceinline__ void pool_walk(const PoolTable<T>* __restrict__ tab, PoolInst<T>& si, long long& sn,
                                          double& svt, int s, Body body) {
    const int ninst = tab->ninst;
    const long long c0 = tab->cls_t0[pool_class(VEC)], c1 = tab->cls_t0[pool_class(VEC) + 1];
    long long lo_t = 0, hi_t = -1;  // tile range of the cached descriptor
    bool run = false;
    for (long long t = c0 + blockIdx.x; t < c1; t += gridDim.x) {
        if (t >= hi_t) {
            __syncthreads();  // the previous descriptor is no longer read
            pool_fetch<T>(tab, ninst, t, &si, &sn, s, &svt);
            __syncthreads();
            lo_t = si.tile0;
            hi_t = si.tile0 + si.ntile;
            run = sn < si.n_end;
        }
        if (run) {
            const long long v = (t - lo_t) * kPoolTpb + threadIdx.x;
            if (v < si.nvec) body(si, v, sn, svt);
        }
    }
}

// Coded two-pass classes with 2- and 4-wide vectors and cell pairs: the first-touch data
// of the same thread's vector (or pair) in the next grid-stride tile (E, H and the code)
// is requested into L2 while this tile is worked on.  Measured on the calibration grids
// (all resident, G cell-updates/s): vec 4 53.7 -> 57.7, vec 2 49.6 -> 60.9; single cells
// 39.4 -> 38.2, so the 1-wide class without pairs (N odd) does without.
#ifndef FIT_POOL_PREFETCH
#define FIT_POOL_PREFETCH 1
#endif
template <typename T, int VEC>
__device__ __forceinline__ void pool_prefetch(const PoolInst<T>& d, long long v, bool e_pass) {
    if constexpr (FIT_POOL_PREFETCH && VEC >= 2) {
        const long long m = (v + (long long)gridDim.x * kPoolTpb) * VEC;
        if (m >= d.g.N) return;
        (void)e_pass;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            prefetch_l2(d.E + c * d.g.N + m);
            prefetch_l2(d.H + c * d.g.N + m);
        }
        prefetch_l2(d.code + m);
    }
}

// MINB: CTAs per SM the register budget is sized for (the launch bound); the pool picks
// one of the compiled variants per vector class.
template <typename T, int VEC, int MINB>
__global__ void __launch_bounds__(kPoolTpb, MINB) k_hpass_pool(const PoolTable<T>* __restrict__ tab, int s) {
    __shared__ PoolInst<T> si;
    __shared__ long long sn;
    __shared__ double svt;
    pool_walk<T, VEC>(tab, si, sn, svt, s, [](const PoolInst<T>& d, long long v, long long, double) {
        if (VEC == 1 && d.pair) {
            pool_prefetch<T, 2>(d, v, false);
            hpass_pair_at<T>(d.E, d.H, d.g, d.mt, v * 2, d.code, d.tab);
        } else if (d.code) {
            pool_prefetch<T, VEC>(d, v, false);
            hpass_at<T, VEC, true>(d.E, d.H, d.ch, d.g, d.mt, v * VEC, d.code, d.tab);
        } else {
            hpass_at<T, VEC>(d.E, d.H, d.ch, d.g, d.mt, v * VEC);
        }
    });
}

template <typename T, int VEC, int MINB>
__global__ void __launch_bounds__(kPoolTpb, MINB) k_epass_pool(const PoolTable<T>* __restrict__ tab, int s) {
    __shared__ PoolInst<T> si;
    __shared__ long long sn;
    __shared__ double svt;
    pool_walk<T, VEC>(tab, si, sn, svt, s, [](const PoolInst<T>& d, long long v, long long n, double vt) {
        StepArgs st{};  // the step and beam position, given
        st.n = n;
        st.vt = vt;
        const PlaneArgs pl{};
        if (VEC == 1 && d.pair) {
            pool_prefetch<T, 2>(d, v, true);
            if (d.mode == 1)
                epass_pair_at<T, 1>(d.E, d.H, d.J, d.use_cond, d.g, d.mt, d.beam, st, v * 2, d.code, d.tab);
            else
                epass_pair_at<T, 0>(d.E, d.H, d.J, d.use_cond, d.g, d.mt, d.beam, st, v * 2, d.code, d.tab);
            return;
        }
        if (d.code) pool_prefetch<T, VEC>(d, v, true);
        if (d.mode == 1 && d.code)
            epass_at<T, VEC, 1, true>(d.E, d.H, d.ce, d.cl, d.J, nullptr, nullptr, d.use_cond, d.g, d.mt, d.beam, pl,
                                      st, v * VEC, d.code, d.tab);
        else if (d.mode == 1)
            epass_at<T, VEC, 1>(d.E, d.H, d.ce, d.cl, d.J, nullptr, nullptr, d.use_cond, d.g, d.mt, d.beam, pl, st,
                                v * VEC);
        else if (d.code)
            epass_at<T, VEC, 0, true>(d.E, d.H, d.ce, d.cl, d.J, nullptr, nullptr, d.use_cond, d.g, d.mt, d.beam, pl,
                                      st, v * VEC, d.code, d.tab);
        else
            epass_at<T, VEC, 0>(d.E, d.H, d.ce, d.cl, d.J, nullptr, nullptr, d.use_cond, d.g, d.mt, d.beam, pl, st,
                                v * VEC);
    });
}

// The fused step of every instance of one fused class, on plane segments.  A work item
// is a segment of S = kSegWin - Nx consecutive cells of the plane-local flat index
// p = i + Nx*j (it spans several rows: a row of these grids is 48-256 cells) and a range
// of zlen planes of one instance; the CTA marches it through the planes.  Per plane k:
//   1. the CTA computes the new H (hpass_eval, the code of every other H update) of a
//      window of kSegWin cells: the segment and the Nx cells before it (plane-local
//      p0-Nx .. p0-1; below p = 0 these are flat-index cells of plane k-1, the -y
//      neighbours the reference's curl couples), every thread the same number of
//      vectors; it stores the window to the plane buffer and the segment to Hout;
//   2. after one barrier each thread updates E of segment cells from the plane buffers
//      of planes k (own, -x and -y neighbours) and k-1 (the -z neighbour).
// Three plane buffers rotate, so one barrier per plane suffices and no value is held in
// registers across it.  A range starting at k0 > 0 first computes the window of plane
// k0-1 (not stored: the range below owns it).  Per cell the step moves E and H once each
// way and a 2-byte coefficient code; the re-reads of neighbours and of the window's
// first Nx cells hit L1/L2.  dir = 0 steps (E, H) -> (E2, H2), dir = 1 back: every
// fused instance enters a chunk with its state in (E, H) and takes an even number of
// steps in it, so all of them share the direction of a step.
template <int VEC>
__host__ __device__ constexpr int seg_reps() {
    return kSegWin / (kSegTpb * VEC);
}

// The instance descriptor lives in shared memory.  Its fields are loop-invariant, and
// the compiler would keep all of them (grid, metric and beam arguments) in registers for
// the whole march; reading the descriptor through an index it cannot see through, once
// per phase, makes it reload them from shared memory instead.
template <typename T>
__device__ __forceinline__ const PoolInst<T>& seg_desc(const PoolInst<T>* dsh) {
    int o = 0;
    asm volatile("" : "+r"(o));
    return dsh[o];
}

// New H of the window of plane k into plane buffer hb[k % 3]; the segment's cells also to
// Hout when store is set.  Window vector u covers plane-local p0 - Nx + u*VEC.
template <typename T, int VEC>
__device__ __forceinline__ void seg_hwindow(const PoolInst<T>& d, const T* __restrict__ Ein,
                                            const T* __restrict__ Hin, T* __restrict__ Hout, long long p0, int k,
                                            bool store, T (*hb)[3][kSegWin]) {
    constexpr int R = seg_reps<VEC>();
    const Geom& g = d.g;
    T(*b)[kSegWin] = hb[k % 3];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int u = threadIdx.x + r * kSegTpb;
        const long long p = p0 - g.nx + (long long)u * VEC;
        if (p >= g.sz) continue;  // past the plane (last segment): never read
        const long long m = p + g.sz * k;
        T ax[VEC], ay[VEC], az[VEC];
        if (m >= 0) {
            int i0, j, kk;
            if (p >= 0) {
                const unsigned q = fdiv((unsigned)p, g.fx);
                j = (int)q;
                i0 = (int)((unsigned)p - q * (unsigned)g.nx);
                kk = k;
            } else {
                cell_of(m, g, i0, j, kk);
            }
            if constexpr (FIT_FUSED_PREFETCH > 0) {
                constexpr int PF = FIT_FUSED_PREFETCH;
                if (store && p >= p0) {  // first-touch data of the segment PF planes ahead
                    if (k + PF + 1 < g.nz) {
                        prefetch_l2(Ein + m + (PF + 1) * g.sz);
                        prefetch_l2(Ein + g.N + m + (PF + 1) * g.sz);
                    }
                    if (k + PF < g.nz) {
                        const long long f = m + PF * g.sz;
                        prefetch_l2(Ein + 2 * g.N + f);
                        prefetch_l2(Hin + f);
                        prefetch_l2(Hin + g.N + f);
                        prefetch_l2(Hin + 2 * g.N + f);
                        prefetch_l2(d.code + f);
                    }
                }
            }
            hpass_eval<T, VEC, true>(Ein, Hin, nullptr, g, d.mt, m, i0, j, kk, ax, ay, az, d.code, d.tab);
            if (store && p >= p0) {
                st_v<T, VEC>(Hout + m, ax);
                st_v<T, VEC>(Hout + g.N + m, ay);
                st_v<T, VEC>(Hout + 2 * g.N + m, az);
            }
        } else {
            zero_v<T, VEC>(ax);
            zero_v<T, VEC>(ay);
            zero_v<T, VEC>(az);
        }
        st_v<T, VEC>(&b[0][u * VEC], ax);
        st_v<T, VEC>(&b[1][u * VEC], ay);
        st_v<T, VEC>(&b[2][u * VEC], az);
    }
}

template <typename T, int VEC, int MODE>
__device__ __forceinline__ void seg_march(const PoolInst<T>* dsh, const T* __restrict__ Ein, const T* __restrict__ Hin,
                                          T* __restrict__ Eout, T* __restrict__ Hout, long long p0, int k0, int k1,
                                          T (*hb)[3][kSegWin], long long step, double vt) {
    constexpr int R = seg_reps<VEC>();
    if (k0 > 0) seg_hwindow<T, VEC>(seg_desc(dsh), Ein, Hin, Hout, p0, k0 - 1, false, hb);
    for (int k = k0; k < k1; ++k) {
        seg_hwindow<T, VEC>(seg_desc(dsh), Ein, Hin, Hout, p0, k, true, hb);
        __syncthreads();
        const PoolInst<T>& d = seg_desc(dsh);
        const Geom& g = d.g;
        const int nx = g.nx;
        T(*b)[kSegWin] = hb[k % 3];
        T(*bm)[kSegWin] = hb[(k + 2) % 3];  // plane k-1
        StepArgs st{};  // the step and beam position, given
        st.n = step;
        st.vt = vt;
        const PlaneArgs pl{};
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int v = threadIdx.x + r * kSegTpb;  // segment vector
            const int x = nx + v * VEC;               // its window column
            const long long p = p0 + (long long)v * VEC;
            if (x >= kSegWin || p >= g.sz) continue;
            const long long n = p + g.sz * k;
            const unsigned q = fdiv((unsigned)p, g.fx);
            const int j = (int)q;
            const int i0 = (int)((unsigned)p - q * (unsigned)nx);
            T hx[VEC], hy[VEC], hz[VEC], hxy[VEC], hzy[VEC], hxz[VEC], hyz[VEC];
            ld_v<T, VEC>(hx, &b[0][x]);
            ld_v<T, VEC>(hy, &b[1][x]);
            ld_v<T, VEC>(hz, &b[2][x]);
            ld_v<T, VEC>(hxy, &b[0][x - nx]);  // n - Nx
            ld_v<T, VEC>(hzy, &b[2][x - nx]);
            const T hyx = b[1][x - 1];  // n - 1
            const T hzx = b[2][x - 1];
            if (k > 0) {
                ld_v<T, VEC>(hxz, &bm[0][x]);  // n - Nx*Ny
                ld_v<T, VEC>(hyz, &bm[1][x]);
            } else {
                zero_v<T, VEC>(hxz);
                zero_v<T, VEC>(hyz);
            }
            T cur[3][VEC];
            epass_curl<T, VEC>(hx, hy, hz, hxy, hzy, hxz, hyz, hyx, hzx, cur, i0, j, k, g, d.mt);
            unsigned cd[VEC];
            ld_codes<VEC>(cd, d.code + n);
            T kx[VEC], ky[VEC], kz[VEC], lx[VEC], ly[VEC], lz[VEC];
            tab_get_v<T, VEC>(d.tab, cd, 1, kx, ky, kz);
            if constexpr (MODE == 1) {
                tab_get_v<T, VEC>(d.tab, cd, 2, lx, ly, lz);
            } else {
                zero_v<T, VEC>(lx);
                zero_v<T, VEC>(ly);
                zero_v<T, VEC>(lz);
            }
            T ex[VEC], ey[VEC], ez[VEC];
            ldg_v<T, VEC>(ex, Ein + n);
            ldg_v<T, VEC>(ey, Ein + g.N + n);
            ldg_v<T, VEC>(ez, Ein + 2 * g.N + n);
            epass_update<T, VEC, MODE>(ex, ey, ez, kx, ky, kz, lx, ly, lz, cur, d.J, n, i0, j, k, d.use_cond, g,
                                       d.beam, pl, st);
            st_v<T, VEC>(Eout + n, ex);
            st_v<T, VEC>(Eout + g.N + n, ey);
            st_v<T, VEC>(Eout + 2 * g.N + n, ez);
        }
    }
}

// MINB: CTAs per SM the register budget is sized for (the launch bound).
template <typename T, int VEC, int MINB>
__global__ void __launch_bounds__(kSegTpb, MINB) k_step_seg_pool(const PoolTable<T>* __restrict__ tab, int dir, int s) {
    __shared__ __align__(16) T hb[3][3][kSegWin];
    __shared__ PoolInst<T> si;
    __shared__ long long sn;
    __shared__ double svt;
    const int ninst = tab->ninst;
    const long long c0 = tab->cls_t0[pool_fused_class(VEC)], c1 = tab->cls_t0[pool_fused_class(VEC) + 1];
    long long lo_w = 0, hi_w = -1;  // work items of the cached descriptor
    bool run = false;
    for (long long w = c0 + blockIdx.x; w < c1; w += gridDim.x) {
        __syncthreads();  // the previous work item no longer reads hb or si
        if (w >= hi_w) {
            pool_fetch<T>(tab, ninst, w, &si, &sn, s, &svt);
            __syncthreads();
            lo_w = si.tile0;
            hi_w = si.tile0 + si.ntile;
            run = sn < si.n_end;
        }
        if (!run) continue;
        const long long local = w - lo_w;
        const int zr = (int)(local / si.nseg);
        const long long p0 = (local - (long long)zr * si.nseg) * (kSegWin - si.g.nx);
        const int k0 = zr * si.zlen, k1 = min(si.g.nz, k0 + si.zlen);
        const T* Ein = dir ? si.E2 : si.E;
        const T* Hin = dir ? si.H2 : si.H;
        T* Eout = dir ? si.E : si.E2;
        T* Hout = dir ? si.H : si.H2;
        if (si.mode == 1)
            seg_march<T, VEC, 1>(&si, Ein, Hin, Eout, Hout, p0, k0, k1, hb, sn, svt);
        else
            seg_march<T, VEC, 0>(&si, Ein, Hin, Eout, Hout, p0, k0, k1, hb, sn, svt);
    }
}

// kPoolProSlices blocks per table row: wake taps of E^n, step n = n0c + s of the row's
// instance (read from the buffer holding the state: the second one on odd steps of a
// fused instance), each block a slice of the step's tap entries; the first block leaves
// the instance's step counter at n + 1, where a later single-grid run continues.  Nothing
// in the pool reads the counter: every pass takes its step from the table.
constexpr int kPoolProSlices = 8;
template <typename T>
__global__ void k_prologue_pool(const PoolTable<T>* __restrict__ tab, int dir, int s) {
    const int row = (int)blockIdx.x / kPoolProSlices, slice = (int)blockIdx.x % kPoolProSlices;
    if (row >= tab->ninst) return;
    const PoolInst<T>& d = tab->inst[row];
    const long long n = d.n0c + s;
    if (n >= d.n_end) return;
    wake_taps<T>((d.fused && dir) ? d.E2 : d.E, d.g, d.tap, n, slice, kPoolProSlices);
    if (slice == 0 && threadIdx.x == 0) *d.d_step = n + 1;
}

}  // namespace fit
