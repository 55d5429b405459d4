// tb_lst.cpp -- linear stability theory (LST) of the Falkner-Skan boundary
// layer for the TS-wave validation of a run (lst_ts/ose_bl.f).
//
// Spatial stability: for real frequency w0 and spanwise wavenumber beta at
// Reynolds number re0 = sqrt(U x / nu), find the complex streamwise
// wavenumber alpha0 of the Orr-Sommerfeld (v) / Squire (vorticity) system,
// written for the oblique wavenumber alpha = sqrt(alpha0^2 + beta^2) with the
// Squire transformation re = re0 alpha0 / alpha, freq = w0 alpha / alpha0.
// The base flow is integrated with the disturbance (f''' = -(m+1)/2 f f''
// - m (1 - f'^2), m = beta_fs / (2 - beta_fs), f''(0) = wslope).
//
//   geom     mapped wall-normal grid eta = L y / (1 - y)          ose_bl.f:419-475
//   derivs   the 21-component ODE: Blasius + 3 solution vectors   ose_bl.f:110-158
//   rkdumb   fixed-step RK4 wall -> eta_max with orthonormalisation (ortho)
//                                                                ose_bl.f:1268-1339, 948-1030
//   deter    6x6 matching determinant with the free-stream decaying
//            solutions exp(-alpha eta), exp(-gamma eta)           ose_bl.f:161-229
//   evalue   secant iteration on alpha (zrtsec)                 ose_bl.f:364-416
//   march    continuation from the starting guess to the target parameters
//            (1000 steps each in Re, omega, beta and the wall shear), then
//            the march over the stations x = 1 + (i-1) dx          ose_bl.f:18-98
// Complex arithmetic follows Fortran complex*16 (library csqrt/cexp/cabs).
#include "tb_internal.h"
#include <array>
#include <cmath>
#include <complex>
#include <vector>

namespace {

typedef std::complex<double> zc;
typedef std::array<zc, 21> V21;
const zc IM(0.0, 1.0);

struct Lst {
    zc re, alfa, alfa0, freq;
    double beta = 0, re0 = 0, w0 = 0, beta_fs = 0;
    double wslope = 0, etamax = 0;
    zc z1, z2, z3, z4;
    int jmax = 0, jedge = 0;
    std::vector<double> eta;
    std::vector<V21> zeig;

    void geom(double bl) {   // ose_bl.f:419-475
        jmax = (int)((double)jedge * bl);
        double dy = 1.0 / (double)(jedge - 1);
        double etal = etamax * (1.0 - (double)(jmax - 1) * dy) / (double)(jmax - 1) / dy;
        eta.assign(jedge + 1, 0.0);
        for (int j = 1; j <= jedge - 1; j++) {
            double y = (double)(j - 1) * dy;
            eta[j] = etal * y / (1.0 - y);
        }
        eta[jmax] = etamax;
        zeig.assign(jmax + 1, V21{});
    }

    void derivs(const V21& zy, V21& zd) const {
        double m = beta_fs / (2.0 - beta_fs);
        zd[0] = zy[1];
        zd[1] = zy[2];
        zd[2] = -zc((m + 1.0) / 2.0) * zy[0] * zy[2] - zc(m) * (zc(1.0) - zy[1] * zy[1]);
        zc utot = zy[1], uptot = zy[2], upptot = zd[2];
        zc z5 = z3 * utot;
        zc z6 = -z1 + z2 * zc(2.0) + z5;
        zc z7 = z4 - z3 * (upptot + z2 * utot);
        zc z8 = -z1 + z2 + z5;
        zc z9 = zc(re0 * beta) * uptot;
        for (int b = 0; b < 3; b++) {   // the three solution vectors at 3, 9, 15
            int o = 3 + 6 * b;
            zd[o] = zy[o + 1];
            zd[o + 1] = zy[o + 2];
            zd[o + 2] = zy[o + 3];
            zd[o + 3] = z6 * zy[o + 2] + z7 * zy[o];
            zd[o + 4] = zy[o + 5];
            zd[o + 5] = z8 * zy[o + 4] + z9 * zy[o];
        }
    }

    void rk4(const V21& zy, const V21& dydx, double h, V21& out) const {   // ose_bl.f:1305-1339
        double hh = h * 0.5, h6 = h / 6.0;
        V21 yt, dyt, dym;
        for (int i = 0; i < 21; i++) yt[i] = zy[i] + zc(hh) * dydx[i];
        derivs(yt, dyt);
        for (int i = 0; i < 21; i++) yt[i] = zy[i] + zc(hh) * dyt[i];
        derivs(yt, dym);
        for (int i = 0; i < 21; i++) { yt[i] = zy[i] + zc(h) * dym[i]; dym[i] = dyt[i] + dym[i]; }
        derivs(yt, dyt);
        for (int i = 0; i < 21; i++) out[i] = zy[i] + zc(h6) * (dydx[i] + dyt[i] + zc(2.0) * dym[i]);
    }

    // Gram-Schmidt of the three solution vectors once they grow (ose_bl.f:948-1030),
    // applied to every stored station below.
    void ortho(V21& zy, int jj) {
        double amag1 = 0, amag2 = 0, amag3 = 0;
        zc g12(0.0), g13(0.0), g23(0.0);
        for (int i = 15; i < 21; i++) {
            amag1 += std::real(zy[i - 12] * std::conj(zy[i - 12]));
            amag2 += std::real(zy[i - 6] * std::conj(zy[i - 6]));
            amag3 += std::real(zy[i] * std::conj(zy[i]));
        }
        amag1 = std::sqrt(amag1); amag2 = std::sqrt(amag2); amag3 = std::sqrt(amag3);
        if (std::max(amag1, std::max(amag2, amag3)) < 50.0 && jj < jmax - 1) return;
        amag1 = 0; amag2 = 0;
        for (int i = 15; i < 21; i++) zy[i] = zy[i] / zc(amag3);
        for (int i = 3; i < 9; i++) { g13 += zy[i] * std::conj(zy[i + 12]); g23 += zy[i + 6] * std::conj(zy[i + 12]); }
        for (int i = 9; i < 15; i++) { zy[i] = zy[i] - g23 * zy[i + 6]; amag2 += std::real(zy[i] * std::conj(zy[i])); }
        amag2 = std::sqrt(amag2);
        for (int i = 9; i < 15; i++) zy[i] = zy[i] / zc(amag2);
        for (int i = 3; i < 9; i++) zy[i] = zy[i] - g13 * zy[i + 12];
        for (int i = 3; i < 9; i++) g12 += zy[i] * std::conj(zy[i + 6]);
        for (int i = 3; i < 9; i++) { zy[i] = zy[i] - g12 * zy[i + 6]; amag1 += std::real(zy[i] * std::conj(zy[i])); }
        amag1 = std::sqrt(amag1);
        for (int i = 3; i < 9; i++) zy[i] = zy[i] / zc(amag1);
        for (int j = 1; j <= jj - 1; j++) {
            V21& z = zeig[j];
            for (int i = 15; i < 21; i++) z[i] = z[i] / zc(amag3);
            for (int i = 9; i < 15; i++) { z[i] = z[i] - g23 * z[i + 6]; z[i] = z[i] / zc(amag2); }
            for (int i = 3; i < 9; i++) { z[i] = z[i] - g13 * z[i + 12] - g12 * z[i + 6]; z[i] = z[i] / zc(amag1); }
        }
    }

    // NR ludcmp with implicit scaling and partial pivoting; returns the determinant.
    static zc det6(zc a[6][6]) {
        const int n = 6;
        double vv[6];
        zc d(1.0);
        for (int i = 0; i < n; i++) {
            double aamax = 0.0;
            for (int j = 0; j < n; j++) aamax = std::max(aamax, std::abs(a[i][j]));
            if (aamax == 0.0) return zc(0.0);
            vv[i] = 1.0 / aamax;
        }
        for (int j = 0; j < n; j++) {
            for (int i = 0; i < j; i++) {
                zc sum = a[i][j];
                for (int k = 0; k < i; k++) sum = sum - a[i][k] * a[k][j];
                a[i][j] = sum;
            }
            double aamax = 0.0;
            int imax = j;
            for (int i = j; i < n; i++) {
                zc sum = a[i][j];
                for (int k = 0; k < j; k++) sum = sum - a[i][k] * a[k][j];
                a[i][j] = sum;
                double dum = vv[i] * std::abs(sum);
                if (dum >= aamax) { imax = i; aamax = dum; }
            }
            if (j != imax) {
                for (int k = 0; k < n; k++) std::swap(a[imax][k], a[j][k]);
                d = -d;
                vv[imax] = vv[j];
            }
            if (a[j][j] == zc(0.0)) a[j][j] = zc(1e-10);
            if (j != n - 1) {
                zc dummy = zc(1.0) / a[j][j];
                for (int i = j + 1; i < n; i++) a[i][j] = a[i][j] * dummy;
            }
        }
        for (int j = 0; j < n; j++) d = d * a[j][j];
        return d;
    }

    zc deter(const V21& zy) const {   // ose_bl.f:161-229
        zc gamma = (freq - alfa) * IM * re;
        gamma = std::sqrt(z2 - gamma);
        double rea = std::real(gamma), aim = std::imag(gamma);
        if (rea < 0.0) rea = -rea;
        if (rea <= 0.0 && aim > 0.0) aim = -aim;
        gamma = zc(rea, aim);
        zc a[6][6];
        for (int r = 0; r < 6; r++) { a[r][0] = zy[3 + r]; a[r][1] = zy[9 + r]; a[r][2] = zy[15 + r]; }
        a[0][3] = zc(-1.0); a[1][3] = alfa; a[2][3] = -alfa * alfa; a[3][3] = alfa * alfa * alfa; a[4][3] = 0.0; a[5][3] = 0.0;
        a[0][4] = zc(-1.0); a[1][4] = gamma; a[2][4] = -gamma * gamma; a[3][4] = gamma * gamma * gamma; a[4][4] = 0.0;
        a[5][4] = 0.0;
        for (int r = 0; r < 4; r++) a[r][5] = 0.0;
        a[4][5] = zc(-1.0); a[5][5] = gamma;
        return det6(a);
    }

    zc init() {   // start + rkdumb + deter (ose_bl.f:478-503, 1230-1301)
        V21 zy{};
        zy[2] = zc(wslope);
        zy[5] = zc(1.0); zy[12] = zc(1.0); zy[20] = zc(1.0);
        zeig[1] = zy;
        V21 dydx, out;
        for (int j = 1; j <= jmax - 1; j++) {
            derivs(zy, dydx);
            double h = eta[j + 1] - eta[j];
            rk4(zy, dydx, h, out);
            zy = out;
            ortho(zy, j + 1);
            zeig[j + 1] = zy;
        }
        return deter(zy);
    }

    // alfa and the constants of derivs; the secant loop forms z3 in the
    // order alfa * i * re, the start in the order i * re * alfa (ose_bl.f:387,402)
    void set_alfa(zc a, bool loop) {
        alfa = a;
        alfa0 = std::sqrt(alfa * alfa - zc(beta * beta));
        re = re0 * alfa0 / alfa;
        freq = w0 * alfa / alfa0;
        z1 = re * IM * freq;
        z2 = alfa * alfa;
        z3 = loop ? alfa * IM * re : IM * re * alfa;
        z4 = z2 * (-z2 + z1);
    }

    // Secant iteration (NR zrtsec) on alfa from the current alfa0 (ose_bl.f:364-416).
    int evalue() {
        zc a1 = std::sqrt(alfa0 * alfa0 + zc(beta * beta));
        alfa = a1;
        re = re0 * alfa0 / alfa;
        freq = w0 * alfa / alfa0;
        z1 = re * IM * freq;
        z2 = alfa * alfa;
        z3 = IM * re * alfa;
        z4 = z2 * (-z2 + z1);
        zc zdet1 = init();
        zc zx1 = alfa, zfl = zdet1;
        set_alfa(zc(1.0001) * a1, false);
        zc zf = init();
        zc zx2 = alfa;
        zc zrtsec, zxl;
        if (std::abs(zfl) < std::abs(zf)) { zrtsec = zx1; zxl = zx2; std::swap(zfl, zf); }
        else { zxl = zx1; zrtsec = zx2; }
        for (int j = 1; j <= 100; j++) {
            zc zdx = (zxl - zrtsec) * zf / (zf - zfl);
            zxl = zrtsec;
            zfl = zf;
            zrtsec = zrtsec + zdx;
            set_alfa(zrtsec, true);
            zf = init();
            double ratr = std::real(zdx) / std::real(zrtsec);
            if (std::fabs(std::imag(zrtsec)) >= 1e-6) {
                double rati = std::imag(zdx) / std::imag(zrtsec);
                if (std::fabs(ratr) <= 5e-5 && std::fabs(rati) <= 1e-2) return TB_OK;
            } else {
                double rati = std::imag(zdx);
                if (std::fabs(ratr) <= 5e-5 && std::fabs(rati) <= 5e-5) return TB_OK;
            }
        }
        tb_set_error("LST: too many secant iterations at re0 = %g", re0);
        return TB_ERR_NOCONV;
    }
};

}  // namespace

extern "C" int tb_lst_march(const tb_lst_config* cf, const double* fpp, const double* betafs, double* x_out,
                            double* re0_out, double* w0_out, double* alpha_out) {
    if (!cf || !fpp || !betafs || !x_out || !re0_out || !w0_out || !alpha_out) { tb_set_error("null argument"); return TB_ERR_ARG; }
    if (cf->jedge < 8 || cf->bl <= 0.0 || cf->bl >= 1.0 || cf->imax < 1 || cf->etamax <= 0.0) {
        tb_set_error("LST: need jedge >= 8, 0 < bl < 1, imax >= 1, etamax > 0");
        return TB_ERR_ARG;
    }
    Lst L;
    L.jedge = cf->jedge;
    L.etamax = cf->etamax;
    L.re0 = cf->re0; L.w0 = cf->w0; L.beta = cf->beta; L.wslope = cf->wslope; L.beta_fs = 0.0;
    L.alfa0 = zc(cf->alfa0_re, cf->alfa0_im);
    L.geom(cf->bl);
    const double w0in = cf->w0, betain = cf->beta, rein0 = cf->re0;
    int r;
    // continuation to the target parameters (ose_bl.f:48-79)
    for (int i = 1; i <= cf->steps; i++) {
        L.re0 = rein0 + (double)(i - 1) * (cf->re_dns - rein0) / (double)cf->steps;
        if ((r = L.evalue())) return r;
    }
    for (int i = 1; i <= cf->steps; i++) {
        L.w0 = w0in + (double)(i - 1) * (cf->omega_dns - w0in) / (double)cf->steps;
        if ((r = L.evalue())) return r;
    }
    for (int i = 1; i <= cf->steps; i++) {
        L.beta = betain + (double)(i - 1) * (cf->beta_dns - betain) / (double)cf->steps;
        if ((r = L.evalue())) return r;
    }
    const double wslopein = L.wslope;
    for (int i = 1; i <= cf->steps; i++) {
        L.wslope = wslopein + (double)(i - 1) * (fpp[0] - wslopein) / (double)cf->steps;
        L.beta_fs = (double)(i - 1) * (betafs[0] - 0.0) / (double)cf->steps;
        if ((r = L.evalue())) return r;
    }
    // march over the stations (ose_bl.f:81-96)
    const double rein = cf->re_dns, w0s = L.w0, betas = L.beta;
    for (int i = 1; i <= cf->imax; i++) {
        double x = 1.0 + (double)(i - 1) * cf->dx;
        L.wslope = fpp[i - 1];
        L.beta_fs = betafs[i - 1];
        L.re0 = rein * std::sqrt(x);
        L.w0 = w0s * L.re0 / rein;
        L.beta = betas * L.re0 / rein;
        if ((r = L.evalue())) return r;
        x_out[i - 1] = (L.re0 / rein) * (L.re0 / rein);
        re0_out[i - 1] = L.re0;
        w0_out[i - 1] = L.w0;
        alpha_out[2 * (i - 1)] = std::real(L.alfa0);
        alpha_out[2 * (i - 1) + 1] = std::imag(L.alfa0);
    }
    return TB_OK;
}
