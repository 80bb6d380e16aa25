// See cell.h.  Follows neighbor_cell.cpp step by step: metric and reduction
// flags (:35-55), 1-D shortest-vector moves (:107-168), inverse axis
// (:170-191), wrap into the cell (:193-200) and translation enumeration
// (:203-253).
#include "cell.h"

#include <cmath>

namespace pg {
namespace {

struct Cell {
    double ax[3][3];  // ax[row][col], columns are lattice vectors
    double d00, d11, d22, d01, d02, d12;
    bool r01, r02, r12;
    int rsum;

    double dot_cols(int a, int b) const {
        return ax[0][a] * ax[0][b] + ax[1][a] * ax[1][b] + ax[2][a] * ax[2][b];
    }
    void metric() {
        d00 = dot_cols(0, 0);
        d11 = dot_cols(1, 1);
        d22 = dot_cols(2, 2);
        d01 = dot_cols(0, 1);
        d02 = dot_cols(0, 2);
        d12 = dot_cols(1, 2);
        r01 = std::fabs(d01) > 0.5 * d00 || std::fabs(d01) > 0.5 * d11;
        r02 = std::fabs(d02) > 0.5 * d00 || std::fabs(d02) > 0.5 * d22;
        r12 = std::fabs(d12) > 0.5 * d11 || std::fabs(d12) > 0.5 * d22;
        rsum = (int)r01 + (int)r02 + (int)r12;
    }
    template <class T>
    void cart(T i, T j, T k, double out[3]) const {
        out[0] = ax[0][0] * i + ax[0][1] * j + ax[0][2] * k;
        out[1] = ax[1][0] * i + ax[1][1] * j + ax[1][2] * k;
        out[2] = ax[2][0] * i + ax[2][1] * j + ax[2][2] * k;
    }
    template <class T>
    double dist(T i, T j, T k) const {
        double v[3];
        cart(i, j, k, v);
        return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    void replace(int i, int j, int k, int col) {
        double v[3];
        cart(i, j, k, v);
        for (int r = 0; r < 3; ++r) ax[r][col] = v[r];
        metric();
    }
    // Each opt_* returns the integer vector of the best 1-D move along one axis.
    void opt0(int v1, int v2, int out[3]) const {
        const double imin = -(d01 * v1 + d02 * v2) / d00;
        out[0] = (int)std::round(imin);
        out[1] = v1;
        out[2] = v2;
    }
    void opt1(int v1, int v2, int out[3]) const {
        const double imin = -(d01 * v1 + d12 * v2) / d11;
        out[0] = v1;
        out[1] = (int)std::round(imin);
        out[2] = v2;
    }
    void opt2(int v1, int v2, int out[3]) const {
        const double imin = -(d02 * v1 + d12 * v2) / d22;
        out[0] = v1;
        out[1] = v2;
        out[2] = (int)std::round(imin);
    }
    void refine() {
        int v[3];
        int iter = 0;
        while (rsum > 0 && iter < 100) {
            if (r01) {
                if (d00 > d11) {
                    opt1(1, 0, v);
                    replace(v[0], v[1], v[2], 0);
                } else {
                    opt0(1, 0, v);
                    replace(v[0], v[1], v[2], 1);
                }
            }
            if (r02) {
                if (d00 > d22) {
                    opt2(1, 0, v);
                    replace(v[0], v[1], v[2], 0);
                } else {
                    opt0(0, 1, v);
                    replace(v[0], v[1], v[2], 2);
                }
            }
            if (r12) {
                if (d11 > d22) {
                    opt2(0, 1, v);
                    replace(v[0], v[1], v[2], 1);
                } else {
                    opt1(0, 1, v);
                    replace(v[0], v[1], v[2], 2);
                }
            }
            ++iter;
        }
    }
    void inverse(double inv[3][3]) const {
        const double(&a)[3][3] = ax;
        const double det = a[0][0] * a[1][1] * a[2][2] + a[0][1] * a[1][2] * a[2][0] +
                           a[0][2] * a[1][0] * a[2][1] - a[0][2] * a[1][1] * a[2][0] -
                           a[0][1] * a[1][0] * a[2][2] - a[0][0] * a[1][2] * a[2][1];
        inv[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
        inv[0][1] = -(a[0][1] * a[2][2] - a[0][2] * a[2][1]);
        inv[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
        inv[1][0] = -(a[1][0] * a[2][2] - a[1][2] * a[2][0]);
        inv[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
        inv[1][2] = -(a[0][0] * a[1][2] - a[0][2] * a[1][0]);
        inv[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
        inv[2][1] = -(a[0][0] * a[2][1] - a[0][1] * a[2][0]);
        inv[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) inv[i][j] /= det;
    }
};

}  // namespace

CellTranslations cell_translations(const double* axis, const double* pos, int n, double cutoff) {
    Cell c;
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) c.ax[r][q] = axis[r * 3 + q];
    c.metric();
    CellTranslations out;
    out.pos.resize(n);
    for (int i = 0; i < n; ++i) out.pos[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    if (c.rsum > 0) {
        c.refine();
        double inv[3][3];
        c.inverse(inv);
        for (int i = 0; i < n; ++i) {
            const double pc[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
            double f[3];
            for (int r = 0; r < 3; ++r) f[r] = inv[r][0] * pc[0] + inv[r][1] * pc[1] + inv[r][2] * pc[2];
            for (int r = 0; r < 3; ++r) f[r] -= std::floor(f[r]);
            double v[3];
            c.cart(f[0], f[1], f[2], v);
            out.pos[i] = {v[0], v[1], v[2]};
        }
    }
    const int e0 = (int)(std::ceil(cutoff / c.dist(1, 0, 0)) + 1);
    const int e1 = (int)(std::ceil(cutoff / c.dist(0, 1, 0)) + 1);
    const int e2 = (int)(std::ceil(cutoff / c.dist(0, 0, 1)) + 1);
    double max_len = 0.0;
    for (int i = -1; i < 2; ++i)
        for (int j = -1; j < 2; ++j)
            for (int k = -1; k < 2; ++k) {
                const double d = c.dist(i, j, k);
                if (max_len < d) max_len = d;
            }
    for (int i = -e0; i < e0 + 1; ++i)
        for (int j = -e1; j < e1 + 1; ++j)
            for (int k = -e2; k < e2 + 1; ++k) {
                double v[3];
                c.cart(i, j, k, v);
                const double d = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (d < max_len + cutoff) {
                    out.trans.push_back({v[0], v[1], v[2]});
                    out.tn.push_back({i, j, k});
                }
            }
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) out.axis[r][q] = c.ax[r][q];
    return out;
}

}  // namespace pg
