// fit_tma.cuh -- the fused leapfrog step fed by tensor-memory-accelerator (TMA) copies.
//
// Same work and arithmetic as k_step_fused (fit_kernels.cuh): a CTA owns a tile of
// FX = 32*VEC cells along x by FY rows along y plus a halo warp, and marches through a
// range of z planes, computing the new H of a plane, then (after one barrier) the new E.
// What changes is how the old fields reach the threads.  Instead of per-thread global
// loads, one thread issues, per plane, three cp.async.bulk.tensor copies into rings of
// shared-memory slots, completion counted on mbarriers:
//   E box  [3 components][FY+2 rows: y0-1 .. y0+FY][EW = FX + 2A: x0-A .. x0+FX+A-1]
//   H box  [3][FY+1 rows: y0-1 .. y0+FY-1][HW = FX + A: x0-A .. x0+FX-1]
//   codes  [FY+1 rows: y0-1 .. y0+FY-1][CW = FX + 8: x0-8 .. x0+FX-1]  (uint16)
// with A = 16 / sizeof(T), so every box starts on a 16-byte boundary along x.  The E box
// holds the tile, the row below (the halo warp's row), the row above (the +y neighbour),
// one column on each side (the -x cell of the halo warp, the +x neighbour), and the
// ring keeps planes k and k+1 (the +z neighbour) while planes up to k+NE-1 are in
// flight; H and codes run NH-1 planes ahead.  Copies out of the grid fill zeros.
//
// The reference's curl couples cells by FLAT index, so the +x neighbour of i = Nx-1 is
// (0, j+1, k), the +y neighbour of j = Ny-1 is (i, 0, k+1), and the cells before a tile
// at x0 = 0 or below a tile at y0 = 0 wrap into the previous row or plane.  Those values
// are not in the box (it holds zeros there); the threads that need them read them from
// global memory, exactly as the direct kernels do, so the inputs of every cell update
// are the same values and the results the same bits as k_step_fused and the two-pass
// kernels (the same hpass_cells / epass_curl / epass_update code computes them).
//
// Waits are bounded (wlim polls): a CTA whose copies do not arrive records
// FIT_ERR_TIMEOUT in *err, stops storing, waits (bounded by kWaitLimit) for the copies it
// issued and returns.  No cluster multicast is used: every copy reads this GPU's own buffers.
#pragma once
#include <cuda.h>

#include "fit_kernels.cuh"

namespace fit {

// 4-D tensor copy (x, y, z, component) global -> shared, completion on an mbarrier
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int c,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(c), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// the same boxes requested into L2 only (no shared memory, no completion to wait for)
__device__ __forceinline__ void tma_prefetch_4d(const CUtensorMap* map, int x, int y, int z, int c) {
    asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(map), "r"(x), "r"(y),
                 "r"(z), "r"(c)
                 : "memory");
}
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* map, int x, int y, int z) {
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(map), "r"(x), "r"(y),
                 "r"(z)
                 : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

// shared-memory layout of one CTA (byte offsets; every slot starts on 128 bytes)
template <typename T, int VEC, int FY, int NE, int NH>
struct TmaLayout {
    static constexpr int FX = 32 * VEC;
    static constexpr int A = 16 / (int)sizeof(T);
    static constexpr int EW = FX + 2 * A;  // E box width (elements)
    static constexpr int HW = FX + A;      // H box width
    static constexpr int CW = FX + 8;      // code box width
    static constexpr int ER = FY + 2;      // E box rows
    static constexpr int HR = FY + 1;      // H and code box rows
    static constexpr unsigned E_BYTES = 3u * ER * EW * sizeof(T);
    static constexpr unsigned H_BYTES = 3u * HR * HW * sizeof(T);
    static constexpr unsigned C_BYTES = (unsigned)HR * CW * 2u;
    static constexpr size_t r128(size_t b) { return (b + 127) / 128 * 128; }
    static constexpr size_t E_SLOT = r128(E_BYTES);
    static constexpr size_t H_SLOT = r128(H_BYTES);
    static constexpr size_t C_SLOT = r128(C_BYTES);
    static constexpr size_t OFF_E = 0;
    static constexpr size_t OFF_H = OFF_E + NE * E_SLOT;
    static constexpr size_t OFF_C = OFF_H + NH * H_SLOT;
    // new H handed between warps: rb[2][Hx, Hz][row][x] -- the row below warp r's row
    // (row 0: the halo warp's row y0-1; row r: warp r-1's row) -- and xb[2][Hy, Hz][row],
    // the cell before each row segment; [2]: ping-pong by plane parity
    static constexpr size_t RB_BYTES = 2u * 2u * FY * FX * sizeof(T);
    static constexpr size_t XB_BYTES = 2u * 2u * FY * sizeof(T);
    static constexpr size_t OFF_R = OFF_C + NH * C_SLOT;
    static constexpr size_t OFF_X = OFF_R + RB_BYTES;
    static constexpr size_t OFF_B = r128(OFF_X + XB_BYTES);
    static constexpr size_t BYTES = OFF_B + (NE + NH) * sizeof(unsigned long long);
    static_assert(EW <= 256 && CW <= 256 && HR + 1 <= 256, "TMA box dimensions are at most 256");
    static_assert((EW * sizeof(T)) % 16 == 0 && (HW * sizeof(T)) % 16 == 0 && (CW * 2) % 16 == 0,
                  "TMA box rows are multiples of 16 bytes");
};

// a vector of VEC values of a box row at column col (16-byte aligned when col*sizeof(T)
// is a multiple of 16)
template <typename T, int VEC>
__device__ __forceinline__ void box_v(T (&r)[VEC], const T* row, int col) {
    ld_v<T, VEC>(r, row + col);
}

// Row-warp / halo-row input gathering for the H update of the VEC cells (i0.., j, k) of
// box row rE (E box) / rH (H and code boxes), box column col (of the first cell, E box
// coordinates; H box column col, code box column col - A + 8).  The +y neighbour of the
// last row (j = Ny-1: the flat crossing into plane k+1) is read from global memory.  The +x
// neighbour after the vector comes from the next lane (shuffle), lane 31 from the box,
// or from global memory at the flat crossing (i0 + VEC = Nx).  Every lane of the warp
// must call this (shuffles); off lanes compute on in-box zeros and store nothing.
template <typename T, int VEC, int FY, int NE, int NH>
__device__ __forceinline__ void tma_hpass_row(const T* __restrict__ Ek, const T* __restrict__ Ek1,
                                              const T* __restrict__ Hk, const unsigned short* __restrict__ Ck,
                                              int rE, int rH, int col, const T* __restrict__ Eg, const Geom& g,
                                              const Metric<T>& mt, const T* __restrict__ tab, long long n, int i0,
                                              int j, int k, int lane, T (&hx)[VEC], T (&hy)[VEC], T (&hz)[VEC],
                                              unsigned (&cd)[VEC]) {
    using L = TmaLayout<T, VEC, FY, NE, NH>;
    constexpr int EW = L::EW, ER = L::ER, HW = L::HW, HR = L::HR, CW = L::CW, A = L::A;
    T ex[VEC], ey[VEC], ez[VEC], exy[VEC], ezy[VEC], exz[VEC], eyz[VEC];
    box_v<T, VEC>(ex, Ek + (0 * ER + rE) * EW, col);
    box_v<T, VEC>(ey, Ek + (1 * ER + rE) * EW, col);
    box_v<T, VEC>(ez, Ek + (2 * ER + rE) * EW, col);
    if (j + 1 < g.ny) {  // warp-uniform
        box_v<T, VEC>(exy, Ek + (0 * ER + rE + 1) * EW, col);
        box_v<T, VEC>(ezy, Ek + (2 * ER + rE + 1) * EW, col);
    } else if (k + 1 < g.nz) {  // flat crossing into plane k+1 (row 0)
        ldg_v<T, VEC>(exy, Eg + n + g.sy);
        ldg_v<T, VEC>(ezy, Eg + 2 * g.N + n + g.sy);
    } else {
        zero_v<T, VEC>(exy);
        zero_v<T, VEC>(ezy);
    }
    if (k + 1 < g.nz) {  // plane k+1; zeros past the last plane, as the direct kernels use
        box_v<T, VEC>(exz, Ek1 + (0 * ER + rE) * EW, col);
        box_v<T, VEC>(eyz, Ek1 + (1 * ER + rE) * EW, col);
    } else {
        zero_v<T, VEC>(exz);
        zero_v<T, VEC>(eyz);
    }
    T eyx = __shfl_down_sync(0xffffffffu, ey[0], 1);
    T ezx = __shfl_down_sync(0xffffffffu, ez[0], 1);
    if (lane == 31) {
        eyx = Ek[(1 * ER + rE) * EW + col + VEC];
        ezx = Ek[(2 * ER + rE) * EW + col + VEC];
    }
    if (i0 + VEC >= g.nx) {  // flat crossing (0, j+1, k) or past the end
        eyx = T(0);
        ezx = T(0);
        if (i0 < g.nx && n + VEC < g.N) {
            eyx = __ldg(Eg + g.N + n + VEC);
            ezx = __ldg(Eg + 2 * g.N + n + VEC);
        }
    }
    const int hcol = col;               // H box starts at x0 - A, like the E box
    const int ccol = col - A + 8;       // code box starts at x0 - 8
    box_v<T, VEC>(hx, Hk + (0 * HR + rH) * HW, hcol);
    box_v<T, VEC>(hy, Hk + (1 * HR + rH) * HW, hcol);
    box_v<T, VEC>(hz, Hk + (2 * HR + rH) * HW, hcol);
    {
        const unsigned short* cp = Ck + rH * CW + ccol;
        if constexpr (VEC == 4) {
            const uint2 t = *reinterpret_cast<const uint2*>(cp);
            cd[0] = t.x & 0xffffu; cd[1] = t.x >> 16; cd[2] = t.y & 0xffffu; cd[3] = t.y >> 16;
        } else if constexpr (VEC == 2) {
            const unsigned t = *reinterpret_cast<const unsigned*>(cp);
            cd[0] = t & 0xffffu; cd[1] = t >> 16;
        } else {
#pragma unroll
            for (int e = 0; e < VEC; ++e) cd[e] = cp[e];
        }
    }
    T cx[VEC], cy[VEC], cz[VEC];
    tab_get_v<T, VEC>(tab, cd, 0, cx, cy, cz);
    hpass_cells<T, VEC>(ex, ey, ez, exy, ezy, exz, eyz, eyx, ezx, hx, hy, hz, cx, cy, cz, i0, j, k, g, mt);
}

// The whole step on coded coefficients (MODE 0 lossless, 1 loss factor): (Ein, Hin) ->
// (Eout, Hout) for the planes [blockIdx.z*zlen, +zlen) of tile column (blockIdx.x,
// blockIdx.y).  tmE / tmH: 4-D maps (Nx, Ny, Nz, 3) of Ein / Hin; tmC: 3-D map of the codes.
// A row warp keeps the new H_x, H_y of its own cells from one plane to the next (the
// plane-below values of the E update); the row-below and cell-before values cross warps
// through the rb / xb buffers, which alternate with the plane parity, so one barrier per
// plane suffices.  MB: CTAs per SM the register budget is sized for.
template <typename T, int VEC, int FY, int MB, int MODE, int NE, int NH>
__global__ void __launch_bounds__(32 * (FY + 1), MB)
    k_step_tma(const __grid_constant__ CUtensorMap tmE, const __grid_constant__ CUtensorMap tmH,
               const __grid_constant__ CUtensorMap tmC, const T* __restrict__ Ein, const T* __restrict__ Hin,
               T* __restrict__ Eout, T* __restrict__ Hout, T* __restrict__ J, int use_cond, Geom g, Metric<T> mt,
               BeamArgs b, StepArgs st, int zlen, const unsigned short* __restrict__ code, const T* __restrict__ tab,
               int* err, long long wlim, int pf) {
    using L = TmaLayout<T, VEC, FY, NE, NH>;
    constexpr int FX = L::FX, A = L::A, EW = L::EW, ER = L::ER, HR = L::HR, HW = L::HW, CW = L::CW;
    extern __shared__ __align__(128) unsigned char smem[];
    T* Ering = reinterpret_cast<T*>(smem + L::OFF_E);
    T* Hring = reinterpret_cast<T*>(smem + L::OFF_H);
    unsigned short* Cring = reinterpret_cast<unsigned short*>(smem + L::OFF_C);
    T(*rb)[2][FY][FX] = reinterpret_cast<T(*)[2][FY][FX]>(smem + L::OFF_R);
    T(*xb)[2][FY] = reinterpret_cast<T(*)[2][FY]>(smem + L::OFF_X);
    unsigned long long* barE = reinterpret_cast<unsigned long long*>(smem + L::OFF_B);
    unsigned long long* barH = barE + NE;

    const int lane = threadIdx.x, ty = threadIdx.y;
    const bool halo = ty == FY;
    const bool producer = halo && lane == 0;
    const int x0 = blockIdx.x * FX, y0 = blockIdx.y * FY;
    const int k0 = blockIdx.z * zlen, k1 = min(g.nz, k0 + zlen);
    const int i0 = x0 + lane * VEC;
    const int j = halo ? y0 - 1 : y0 + ty;  // the halo warp's own row is the one below the tile
    const bool on = i0 < g.nx && j >= 0 && j < g.ny;
    const int xo = lane * VEC;
    const PlaneArgs pl{};

    auto eslot = [&](int p) { return Ering + (size_t)((p - k0) % NE) * (L::E_SLOT / sizeof(T)); };
    auto hslot = [&](int p) { return Hring + (size_t)((p - k0) % NH) * (L::H_SLOT / sizeof(T)); };
    auto cslot = [&](int p) { return Cring + (size_t)((p - k0) % NH) * (L::C_SLOT / 2); };
    auto issue_e = [&](int p) {
        unsigned long long* bar = &barE[(p - k0) % NE];
        mbar_arrive_tx(bar, L::E_BYTES);
        tma_load_4d(eslot(p), &tmE, x0 - A, y0 - 1, p, 0, bar);
    };
    auto issue_h = [&](int p) {
        unsigned long long* bar = &barH[(p - k0) % NH];
        mbar_arrive_tx(bar, L::H_BYTES + L::C_BYTES);
        tma_load_4d(hslot(p), &tmH, x0 - A, y0 - 1, p, 0, bar);
        tma_load_3d(cslot(p), &tmC, x0 - 8, y0 - 1, p, bar);
    };

    if (producer) {
        prefetch_tmap(&tmE);
        prefetch_tmap(&tmH);
        prefetch_tmap(&tmC);
        for (int s = 0; s < NE + NH; ++s) mbar_init(&barE[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // E planes k0 .. e_last (plane k1 is the +z neighbour of the range's last plane; none
    // past the grid), H and code planes k0 .. k1-1
    const int e_last = min(k1, g.nz - 1);
    int e_issued = k0 - 1, h_issued = k0 - 1;  // last plane issued (producer only)
    if (producer) {
        for (int p = k0; p <= min(e_last, k0 + NE - 2); ++p) issue_e(p);
        e_issued = min(e_last, k0 + NE - 2);
        for (int p = k0; p <= min(k1 - 1, k0 + NH - 2); ++p) issue_h(p);
        h_issued = min(k1 - 1, k0 + NH - 2);
        // L2 prefetch of the planes the next pf ring loads will read
        for (int p = e_issued + 1; p <= min(e_last, e_issued + pf); ++p) tma_prefetch_4d(&tmE, x0 - A, y0 - 1, p, 0);
        for (int p = h_issued + 1; p <= min(k1 - 1, h_issued + pf); ++p) {
            tma_prefetch_4d(&tmH, x0 - A, y0 - 1, p, 0);
            tma_prefetch_3d(&tmC, x0 - 8, y0 - 1, p);
        }
    }
    // the new H_x, H_y of the thread's cells one plane below (zero below plane 0); for a
    // range starting at k0 > 0, plane k0-1 computed from global memory (the CTA below
    // stores it)
    T px[VEC], py[VEC];
    zero_v<T, VEC>(px);
    zero_v<T, VEC>(py);
    if (k0 > 0 && !halo && on) {
        T hz[VEC];
        const long long n = (long long)i0 + g.sy * j + g.sz * (k0 - 1);
        hpass_eval<T, VEC, true>(Ein, Hin, nullptr, g, mt, n, i0, j, k0 - 1, px, py, hz, code, tab);
    }
    bool ok = mbar_wait(&barE[0], 0u, wlim);  // plane k0 of E
    int kdone = k0;                            // planes [k0, kdone) completed
    for (int k = k0; k < k1; ++k) {
        const int bc = k & 1;
        if (k + 1 <= e_last)
            ok = ok && mbar_wait(&barE[(k + 1 - k0) % NE], (unsigned)(((k + 1 - k0) / NE) & 1), wlim);
        ok = ok && mbar_wait(&barH[(k - k0) % NH], (unsigned)(((k - k0) / NH) & 1), wlim);
        const T* Ek = eslot(k);
        const T* Ek1 = eslot(k + 1);
        const T* Hk = hslot(k);
        const unsigned short* Ck = cslot(k);
        const long long n = (long long)i0 + g.sy * j + g.sz * k;
        T hx[VEC], hy[VEC], hz[VEC];
        unsigned cd[VEC];
        if (!halo) {
            if (j < g.ny) {  // warp-uniform
                tma_hpass_row<T, VEC, FY, NE, NH>(Ek, Ek1, Hk, Ck, ty + 1, ty + 1, A + xo, Ein, g, mt, tab, n, i0, j,
                                                  k, lane, hx, hy, hz, cd);
                if (on && ok) {
                    st_v<T, VEC>(Hout + n, hx);
                    st_v<T, VEC>(Hout + g.N + n, hy);
                    st_v<T, VEC>(Hout + 2 * g.N + n, hz);
                }
                if (ty + 1 < FY) {  // the row below of warp ty+1
                    st_v<T, VEC>(&rb[bc][0][ty + 1][xo], hx);
                    st_v<T, VEC>(&rb[bc][1][ty + 1][xo], hz);
                }
            }
        } else {
            // the row below the tile: flat n - Nx
            if (y0 > 0) {
                T ax[VEC], ay[VEC], az[VEC];
                unsigned cq[VEC];
                tma_hpass_row<T, VEC, FY, NE, NH>(Ek, Ek1, Hk, Ck, 0, 0, A + xo, Ein, g, mt, tab, n, i0, j, k, lane,
                                                  ax, ay, az, cq);
                st_v<T, VEC>(&rb[bc][0][0][xo], ax);
                st_v<T, VEC>(&rb[bc][1][0][xo], az);
            } else if (i0 < g.nx) {  // y0 = 0: wraps to (i, Ny-1, k-1)
                T ax[VEC], ay[VEC], az[VEC];
                const long long m = (long long)i0 + g.sz * k - g.sy;
                if (m >= 0) {
                    int mi, mj, mk;
                    cell_of(m, g, mi, mj, mk);
                    hpass_eval<T, VEC, true>(Ein, Hin, nullptr, g, mt, m, mi, mj, mk, ax, ay, az, code, tab);
                } else {
                    zero_v<T, VEC>(ax);
                    zero_v<T, VEC>(az);
                }
                st_v<T, VEC>(&rb[bc][0][0][xo], ax);
                st_v<T, VEC>(&rb[bc][1][0][xo], az);
            }
            // the cell before each row segment: flat n - 1
            const int jj = y0 + lane;
            if (lane < FY && jj < g.ny) {
                T ax[1], ay[1], az[1];
                const long long m = (long long)x0 + g.sy * jj + g.sz * k - 1;
                if (x0 > 0) {  // (x0-1, jj, k): in the boxes
                    const int r = lane + 1, c0 = A - 1;
                    T ex1[1] = {Ek[(0 * ER + r) * EW + c0]}, ey1[1] = {Ek[(1 * ER + r) * EW + c0]},
                      ez1[1] = {Ek[(2 * ER + r) * EW + c0]};
                    T exy1[1], ezy1[1];
                    if (jj + 1 < g.ny) {
                        exy1[0] = Ek[(0 * ER + r + 1) * EW + c0];
                        ezy1[0] = Ek[(2 * ER + r + 1) * EW + c0];
                    } else if (k + 1 < g.nz) {
                        exy1[0] = __ldg(Ein + m + g.sy);
                        ezy1[0] = __ldg(Ein + 2 * g.N + m + g.sy);
                    } else {
                        exy1[0] = T(0);
                        ezy1[0] = T(0);
                    }
                    T exz1[1] = {T(0)}, eyz1[1] = {T(0)};
                    if (k + 1 < g.nz) {
                        exz1[0] = Ek1[(0 * ER + r) * EW + c0];
                        eyz1[0] = Ek1[(1 * ER + r) * EW + c0];
                    }
                    const T eyx1 = Ek[(1 * ER + r) * EW + c0 + 1], ezx1 = Ek[(2 * ER + r) * EW + c0 + 1];
                    ax[0] = Hk[(0 * HR + r) * HW + c0];
                    ay[0] = Hk[(1 * HR + r) * HW + c0];
                    az[0] = Hk[(2 * HR + r) * HW + c0];
                    unsigned c1[1] = {Ck[r * CW + 7]};
                    T cx[1], cy[1], cz[1];
                    tab_get_v<T, 1>(tab, c1, 0, cx, cy, cz);
                    hpass_cells<T, 1>(ex1, ey1, ez1, exy1, ezy1, exz1, eyz1, eyx1, ezx1, ax, ay, az, cx, cy, cz,
                                      x0 - 1, jj, k, g, mt);
                } else if (m >= 0) {  // x0 = 0: wraps to (Nx-1, jj-1, k) or further
                    int mi, mj, mk;
                    cell_of(m, g, mi, mj, mk);
                    hpass_eval<T, 1, true>(Ein, Hin, nullptr, g, mt, m, mi, mj, mk, ax, ay, az, code, tab);
                } else {
                    ay[0] = T(0);
                    az[0] = T(0);
                }
                xb[bc][0][lane] = ay[0];
                xb[bc][1][lane] = az[0];
            }
        }
        // every thread is past plane k-1 (its ring slots and the rb / xb buffers of plane
        // k+1's parity are free) and the new H of plane k is in rb / xb; the give-up
        // decision is CTA-uniform
        ok = __syncthreads_and(ok);
        if (!ok) break;
        kdone = k + 1;
        if (producer) {
            fence_proxy_async();
            if (e_issued < e_last && e_issued + 1 <= k + NE - 1) issue_e(++e_issued);
            if (h_issued < k1 - 1 && h_issued + 1 <= k + NH - 1) issue_h(++h_issued);
            // keep the L2 prefetch pf planes ahead of the ring loads
            if (pf > 0 && e_issued + pf <= e_last) tma_prefetch_4d(&tmE, x0 - A, y0 - 1, e_issued + pf, 0);
            if (pf > 0 && h_issued + pf <= k1 - 1) {
                tma_prefetch_4d(&tmH, x0 - A, y0 - 1, h_issued + pf, 0);
                tma_prefetch_3d(&tmC, x0 - 8, y0 - 1, h_issued + pf);
            }
        }
        if (!halo && j < g.ny) {
            T hxy[VEC], hzy[VEC];
            ld_v<T, VEC>(hxy, &rb[bc][0][ty][xo]);
            ld_v<T, VEC>(hzy, &rb[bc][1][ty][xo]);
            T hyx = __shfl_up_sync(0xffffffffu, hy[VEC - 1], 1);
            T hzx = __shfl_up_sync(0xffffffffu, hz[VEC - 1], 1);
            if (lane == 0) {
                hyx = xb[bc][0][ty];
                hzx = xb[bc][1][ty];
            }
            T cur[3][VEC];
            epass_curl<T, VEC>(hx, hy, hz, hxy, hzy, px, py, hyx, hzx, cur, i0, j, k, g, mt);
            T kx[VEC], ky[VEC], kz[VEC], lx[VEC], ly[VEC], lz[VEC];
            tab_get_v<T, VEC>(tab, cd, 1, kx, ky, kz);
            if constexpr (MODE == 1) {
                tab_get_v<T, VEC>(tab, cd, 2, lx, ly, lz);
            } else {
                zero_v<T, VEC>(lx);
                zero_v<T, VEC>(ly);
                zero_v<T, VEC>(lz);
            }
            T ex[VEC], ey[VEC], ez[VEC];
            box_v<T, VEC>(ex, Ek + (0 * ER + ty + 1) * EW, A + xo);
            box_v<T, VEC>(ey, Ek + (1 * ER + ty + 1) * EW, A + xo);
            box_v<T, VEC>(ez, Ek + (2 * ER + ty + 1) * EW, A + xo);
            if (on) {
                epass_update<T, VEC, MODE>(ex, ey, ez, kx, ky, kz, lx, ly, lz, cur, J, n, i0, j, k, use_cond, g, b, pl,
                                           st);
                st_v<T, VEC>(Eout + n, ex);
                st_v<T, VEC>(Eout + g.N + n, ey);
                st_v<T, VEC>(Eout + 2 * g.N + n, ez);
            }
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                px[e] = hx[e];
                py[e] = hy[e];
            }
        }
    }
    if (!ok && producer) {
        atomicExch(err, FIT_ERR_TIMEOUT);
        // bounded waits for the copies issued and not consumed, so none lands after exit
        for (int p = kdone + 1; p <= e_issued; ++p)
            mbar_wait(&barE[(p - k0) % NE], (unsigned)(((p - k0) / NE) & 1), kWaitLimit);
        for (int p = kdone; p <= h_issued; ++p)
            mbar_wait(&barH[(p - k0) % NH], (unsigned)(((p - k0) / NH) & 1), kWaitLimit);
    }
}

}  // namespace fit
