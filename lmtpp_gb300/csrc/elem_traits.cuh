// elem_traits.cuh -- reference-cell data of the element types on the path (shape-function
// derivatives and Gauss rules), shared by the element-matrix and gradient kernels.
//
//   Hexa8    trilinear on [0,1]^3 (formulations/element_Hexa.py:61-68); order-2 rule of the
//            reference table: 2x2x2 points, 12-significant-digit abscissae 0.211324865405 /
//            0.788675134595, weights 1/8 (include/mesh/element_Hexa.h:5-20)
//   Tetra10  quadratic on the unit tetrahedron (formulations/element_Tetra_10.py:27-41), node
//            order 0-3 vertices, 4:(0,1) 5:(1,2) 6:(0,2) 7:(0,3) 8:(1,3) 9:(2,3); order-2 rule:
//            4 points, abscissae 0.1381966011250105 / 0.5854101966249685, weights 1/24
//            (include/mesh/element_Tetra_10.h:5-16)
#pragma once
#include "lmtg_internal.cuh"

namespace lmtg {

struct Hexa8 {
    static constexpr int npe = 8, ngp = 8, npairs = 36;
    template <class T>
    __host__ __device__ static T weight(int) { return (T)0.125; }
    template <class T>
    __host__ __device__ static void dN(int g, T (&d)[8][3]) {
        const T ga = (T)0.211324865405, gb = (T)0.788675134595;
        const T x = (g == 1 || g == 2 || g == 5 || g == 6) ? gb : ga;
        const T y = (g == 2 || g == 3 || g == 6 || g == 7) ? gb : ga;
        const T z = (g >= 4) ? gb : ga;
        dN_at(x, y, z, d);
    }
    // shape functions at the reference point (x, y, z)
    template <class T>
    __device__ static void N_at(T x, T y, T z, T (&N)[8]) {
        const T mx = 1 - x, my = 1 - y, mz = 1 - z;
        N[0] = mx * my * mz; N[1] = x * my * mz; N[2] = x * y * mz; N[3] = mx * y * mz;
        N[4] = mx * my * z;  N[5] = x * my * z;  N[6] = x * y * z;  N[7] = mx * y * z;
    }
    // Gauss point g of the order-2 rule
    template <class T>
    __host__ __device__ static void gauss_point(int g, T &x, T &y, T &z) {
        const T ga = (T)0.211324865405, gb = (T)0.788675134595;
        x = (g == 1 || g == 2 || g == 5 || g == 6) ? gb : ga;
        y = (g == 2 || g == 3 || g == 6 || g == 7) ? gb : ga;
        z = (g >= 4) ? gb : ga;
    }
    // derivatives at the reference point (x, y, z)
    template <class T>
    __host__ __device__ static void dN_at(T x, T y, T z, T (&d)[8][3]) {
        const T mx = 1 - x, my = 1 - y, mz = 1 - z;
        d[0][0] = -my * mz; d[0][1] = -mx * mz; d[0][2] = -mx * my;
        d[1][0] = my * mz;  d[1][1] = -x * mz;  d[1][2] = -x * my;
        d[2][0] = y * mz;   d[2][1] = x * mz;   d[2][2] = -x * y;
        d[3][0] = -y * mz;  d[3][1] = mx * mz;  d[3][2] = -mx * y;
        d[4][0] = -my * z;  d[4][1] = -mx * z;  d[4][2] = mx * my;
        d[5][0] = my * z;   d[5][1] = -x * z;   d[5][2] = x * my;
        d[6][0] = y * z;    d[6][1] = x * z;    d[6][2] = x * y;
        d[7][0] = -y * z;   d[7][1] = mx * z;   d[7][2] = mx * y;
    }
};

struct Tetra10 {
    static constexpr int npe = 10, ngp = 4, npairs = 55;
    template <class T>
    __host__ __device__ static T weight(int) { return (T)0.041666666666666666667; }
    template <class T>
    __host__ __device__ static void dN(int g, T (&d)[10][3]) {
        const T ta = (T)0.1381966011250105, tb = (T)0.5854101966249685;
        const T x = g == 1 ? tb : ta, y = g == 2 ? tb : ta, z = g == 3 ? tb : ta;
        dN_at(x, y, z, d);
    }
    template <class T>
    __device__ static void N_at(T x, T y, T z, T (&N)[10]) {
        const T X[4] = {1 - x - y - z, x, y, z};
#pragma unroll
        for (int i = 0; i < 4; ++i) N[i] = X[i] * (2 * X[i] - 1);
        N[4] = 4 * X[0] * X[1]; N[5] = 4 * X[1] * X[2]; N[6] = 4 * X[0] * X[2];
        N[7] = 4 * X[0] * X[3]; N[8] = 4 * X[1] * X[3]; N[9] = 4 * X[2] * X[3];
    }
    template <class T>
    __host__ __device__ static void gauss_point(int g, T &x, T &y, T &z) {
        const T ta = (T)0.1381966011250105, tb = (T)0.5854101966249685;
        x = g == 1 ? tb : ta;
        y = g == 2 ? tb : ta;
        z = g == 3 ? tb : ta;
    }
    // derivatives at the reference point (x, y, z)
    template <class T>
    __host__ __device__ static void dN_at(T x, T y, T z, T (&d)[10][3]) {
        const T X0 = 1 - x - y - z, X1 = x, X2 = y, X3 = z;
        // vertices: d(Xi (2 Xi - 1)) = (4 Xi - 1) dXi, dX0 = (-1,-1,-1)
        const T c0 = 4 * X0 - 1;
        d[0][0] = -c0; d[0][1] = -c0; d[0][2] = -c0;
        d[1][0] = 4 * X1 - 1; d[1][1] = 0; d[1][2] = 0;
        d[2][0] = 0; d[2][1] = 4 * X2 - 1; d[2][2] = 0;
        d[3][0] = 0; d[3][1] = 0; d[3][2] = 4 * X3 - 1;
        // edges 4 Xa Xb
        d[4][0] = 4 * (X0 - X1); d[4][1] = -4 * X1; d[4][2] = -4 * X1;           // (0,1)
        d[5][0] = 4 * X2; d[5][1] = 4 * X1; d[5][2] = 0;                           // (1,2)
        d[6][0] = -4 * X2; d[6][1] = 4 * (X0 - X2); d[6][2] = -4 * X2;           // (0,2)
        d[7][0] = -4 * X3; d[7][1] = -4 * X3; d[7][2] = 4 * (X0 - X3);           // (0,3)
        d[8][0] = 4 * X3; d[8][1] = 0; d[8][2] = 4 * X1;                           // (1,3)
        d[9][0] = 0; d[9][1] = 4 * X3; d[9][2] = 4 * X2;                           // (2,3)
    }
};

}  // namespace lmtg
