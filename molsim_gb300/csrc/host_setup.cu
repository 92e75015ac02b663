// host_setup.cu — host-side set-up of the hot path (once per parameter set).
//
//  * the two-body table of the (1,6,12) + Ewald-real-space potential
//    (PotTwoBodyTab1/2/3, SetUBuffer, CheckUBuffer: potential.F90:868-1263;
//    Pot_1_6_12 potential.F90:1349-1434; CalcEwaldUfac potential.F90:2938;
//    Erf2 mollib.F90:215-274),
//  * RcutToAlpha (energy.F90:7090-7106),
//  * the SPME influence tables and the standard-Ewald k-vectors
//    (EwaldSetup, energy.F90:6640-7018),
//  * the cardinal B-spline (mollib.F90:1629-1685).
//
// All of it is double precision on the host and compiled without FMA
// contraction (-ffp-contract=off), so the table, the tables' interval ends and
// the Ewald factors carry exactly the bits the reference's expressions give.
#include <cmath>
#include <cstring>
#include <vector>

#include "mg_erf.cuh"
#include "mg_internal.cuh"

namespace {

const double kPi = 3.1415926535897932;   // mol.F90:63

// x**n as gfortran -O2 expands it for the powers used here
inline double sq(double x) { return x * x; }
inline double cube(double x) { return (x * x) * x; }
inline double sixth(double x) {
    double x3 = (x * x) * x;
    return x3 * x3;
}

// Erf2 (mollib.F90:215-274), shared with the device code
double erf_reference(double x) { return mg_erf2(x); }

struct Potential {
    const mg_pot_params &pp;
    // u0 = u(r), u1 = du/dr, u2 = d2u/dr2 for the type pair (i, j), 1-based
    void eval(int i, int j, double r1, double &u0, double &u1, double &u2) const {
        double qq = pp.zat[i - 1] * pp.zat[j - 1] * pp.epsi_four_pi;
        double sig = 0.5 * (pp.sigat[i - 1] + pp.sigat[j - 1]);
        double eps = std::sqrt(pp.epsat[i - 1] * pp.epsat[j - 1]);
        double r1i = 1.0 / r1;
        double fac = sixth(sig * r1i);
        double c0 = 1.0, c1 = 1.0, c2 = 1.0;
        if (pp.lcharge_ewald) {
            const double f = 1.12837916709;
            double ra = pp.ualpha * r1;
            double er = erf_reference(ra);
            double ex = f * std::exp(-(ra * ra));
            c0 = 1.0 - (er);
            c1 = 1.0 - (er - ra * ex);
            c2 = 1.0 - (er - ra * (1.0 + ra * ra) * ex);
        }
        double s0 = +4.0 * eps * (fac * fac - fac);
        double s1 = -(24.0 * eps * (2.0 * (fac * fac) - fac) * r1i);
        double s2 = +24.0 * eps * (26.0 * (fac * fac) - 7.0 * fac) * (r1i * r1i);
        if (pp.lljcut) {
            if (r1 < pp.ljrcut * sig) {
                s0 = s0 + pp.ljushift * eps;
            } else {
                s0 = 0.0;
                s1 = 0.0;
                s2 = 0.0;
            }
        }
        u0 = qq * c0 * r1i + s0;
        u1 = -(qq * c1 * (r1i * r1i)) + s1;
        u2 = 2.0 * qq * c2 * cube(r1i) + s2;
    }
};

// quintic in z = r^2 through (u, u', u'') at both ends (SetUBuffer)
void fit_interval(double zlo, double u0l, double u1l, double u2l, double zhi, double u0h,
                  double u1h, double u2h, double *rec) {
    if (u0l == 0.0 && u0h == 0.0) {
        rec[0] = zlo;
        for (int i = 1; i < 12; ++i) rec[i] = 0.0;
        return;
    }
    double rlo = std::sqrt(zlo), rhi = std::sqrt(zhi);
    double dz1 = zhi - zlo, dz2 = dz1 * dz1, dz3 = dz2 * dz1;
    double w0l = u0l, w0h = u0h;
    double w1l = 0.50 * u1l / rlo, w1h = 0.50 * u1h / rhi;
    double w2l = 0.25 * (u2l - u1l / rlo) / zlo, w2h = 0.25 * (u2h - u1h / rhi) / zhi;
    double a = 6.0 * (w0h - w0l - w1l * dz1 - 0.5 * w2l * dz2) / dz3;
    double b = 2.0 * (w1h - w1l - w2l * dz1) / dz2;
    double c = (w2h - w2l) / dz1;
    rec[0] = zlo;
    rec[1] = w0l;
    rec[2] = w1l;
    rec[3] = 0.5 * w2l;
    rec[4] = (10.0 * a - 12.0 * b + 3.0 * c) / (6.0);
    rec[5] = (-15.0 * a + 21.0 * b - 6.0 * c) / (6.0 * dz1);
    rec[6] = (2.0 * a - 3.0 * b + c) / (2.0 * dz2);
    rec[7] = -2.0 * rec[2];
    rec[8] = -4.0 * rec[3];
    rec[9] = -6.0 * rec[4];
    rec[10] = -8.0 * rec[5];
    rec[11] = -10.0 * rec[6];
}

// CheckUBuffer: 11 equidistant points in r against utoltab/ftoltab
void check_interval(const Potential &pot, int i, int j, double rlo, double rhi, const double *rec,
                    bool &ok, bool &repul) {
    const mg_pot_params &pp = pot.pp;
    ok = false;
    repul = false;
    double dr = (rhi - rlo) / (11 - 1);
    for (int k = 1; k <= 11; ++k) {
        double r1 = rlo + dr * (k - 1), u0, u1, u2;
        pot.eval(i, j, r1, u0, u1, u2);
        double dz = r1 * r1 - rlo * rlo;
        double us = rec[1] + dz * (rec[2] + dz * (rec[3] + dz * (rec[4] + dz * (rec[5] + dz * rec[6]))));
        double fs = rec[7] + dz * (rec[8] + dz * (rec[9] + dz * (rec[10] + dz * rec[11])));
        fs = r1 * fs;
        if (std::fabs(us - u0) > pp.utoltab) return;
        if (std::fabs(fs + u1) > pp.ftoltab) return;
        if (std::fabs(us) > pp.umaxtab) repul = true;
        if (std::fabs(fs) > pp.fmaxtab) repul = true;
    }
    ok = true;
}

}  // namespace

// PotTwoBodyTab1 -> Tab2 -> Tab3 for every type pair, in the reference's order
// (ipt = 1..npt, jpt = ipt..npt), intervals from rumax = 1.1 rcut downwards.
int mg_host_table(const mg_pot_params *pp, double *ubuf, int32_t nbuf_cap, int32_t *nbuf_used,
                  int32_t *iubuflow, double *r2umin, int32_t *nugrid) {
    if (!pp || pp->npt < 1 || !nbuf_used || !iubuflow || !r2umin || !nugrid) return MG_ERR_ARG;
    const int max_intervals = 1200, max_tries = 100;
    const double shrink = 0.9;
    Potential pot{*pp};
    int npt = pp->npt, nptpt = npt * (npt + 1) / 2;
    std::vector<double> table;
    std::vector<char> done(nptpt, 0);
    int status = MG_OK;
    for (int i = 1; i <= npt && status == MG_OK; ++i) {
        for (int j = i; j <= npt && status == MG_OK; ++j) {
            int pair = pp->iptpt[(j - 1) * npt + (i - 1)];
            if (pair < 1 || pair > nptpt) return MG_ERR_ARG;
            if (done[pair - 1]) continue;
            double rmax = std::sqrt(sq(1.1 * (pp->rcut + 0.0 + 0.0)));
            double rmin = std::sqrt(pp->r2uminin);
            iubuflow[pair - 1] = (int32_t)table.size() + 1;
            double rhi = rmax, dr = 0.5 * (rmax - rmin), rlo = 0.0;
            int n = 0;
            bool finished = false;
            for (n = 1; n <= max_intervals; ++n) {
                double zhi = rhi * rhi, rec[12];
                bool ok = false, repul = false;
                int tries;
                for (tries = 1; tries <= max_tries; ++tries) {
                    rlo = rhi - dr;
                    rlo = (rmin > rlo) ? rmin : rlo;
                    double zlo = rlo * rlo, a0, a1, a2, b0, b1, b2;
                    pot.eval(i, j, rlo, a0, a1, a2);
                    pot.eval(i, j, rhi, b0, b1, b2);
                    fit_interval(zlo, a0, a1, a2, zhi, b0, b1, b2, rec);
                    check_interval(pot, i, j, rlo, rhi, rec, ok, repul);
                    if (ok) {
                        rhi = rlo;
                        if (pp->lljcut) dr = 2.0 * dr;
                        break;
                    }
                    dr = dr * shrink;
                }
                if (tries > max_tries) {
                    status = MG_ERR_TABLE;
                    break;
                }
                table.insert(table.end(), rec, rec + 12);
                if (repul) rmin = rlo;
                if (rlo <= rmin || repul) {
                    finished = true;
                    break;
                }
            }
            if (status != MG_OK) break;
            if (!finished) {
                status = MG_ERR_TABLE;
                break;
            }
            nugrid[pair - 1] = n;
            r2umin[pair - 1] = rmin * rmin;
            done[pair - 1] = 1;
        }
    }
    *nbuf_used = (int32_t)table.size();
    if (status != MG_OK) return status;
    if (!ubuf || (int64_t)table.size() > nbuf_cap) return MG_ERR_TABLE;
    std::memcpy(ubuf, table.data(), sizeof(double) * table.size());
    return MG_OK;
}

int mg_host_rcut_to_alpha(double tol, double rcut, double q2sum, double L, double efp,
                          double *ualpha) {
    if (!(tol > 0) || !(rcut > 0) || !(q2sum > 0) || !ualpha) return MG_ERR_ARG;
    double y = (tol / (q2sum * efp)) * std::sqrt(2.0 * cube(L * rcut));
    double xold = 1.0e-1, xnew = 0.0;
    for (int i = 1; i <= 40; ++i) {
        xnew = (1.0 / rcut) * std::sqrt(-std::log(y * (xold * xold)));
        if (std::fabs(xold - xnew) / xnew < 1.0e-6) {
            *ualpha = xnew;
            return MG_OK;
        }
        xold = xnew;
    }
    return MG_ERR_ARG;
}

int mg_host_bspline(int order, double pos, int *kmax, double *v, double *dv) {
    double last[MG_MAX_ORDER];
    if (order < 1 || order > MG_MAX_ORDER) return MG_ERR_ARG;
    int k = (int)std::floor(pos);
    double x = pos - k;
    *kmax = k;
    for (int i = 0; i < order; ++i) last[i] = 0.0;
    v[0] = x;
    if (order > 1) {
        v[1] = 1.0 - x;
        for (int n = 3; n <= order; ++n) {
            for (int i = 0; i < order; ++i) last[i] = v[i];
            v[0] = x * last[0] / (n - 1);
            for (int i = 1; i <= n - 2; ++i) {
                double a = i + x;
                v[i] = (a * last[i] + (n - a) * last[i - 1]) / (n - 1);
            }
            v[n - 1] = (1 - x) * last[n - 2] / (n - 1);
        }
        if (dv) {
            dv[0] = last[0];
            for (int i = 1; i <= order - 2; ++i) dv[i] = last[i] - last[i - 1];
            dv[order - 1] = -last[order - 2];
        }
    }
    return MG_OK;
}

// Influence tables on the octant [0, n/2]^3, stored [fz][fy][kx] (kx fastest):
//   mf = meshfac as EwaldSetup computes it (energy.F90:6996-7018);
//   ew, vw = energyfac, virfac with the halving for the y and z self-mirror
//   planes undone, because the device visits every half-spectrum point once
//   instead of the reference's four-fold (ny, nz) mirror walk in SPMFFTRec;
//   the kx = 0, n/2 halving is kept.
void mg_host_spme_tables(int n, int order, const double boxlen[3], const double TwoPiBoxi[3],
                         double vol, double ualpha, std::vector<double> &mf, std::vector<double> &ew,
                         std::vector<double> &vw) {
    int nh = n / 2 + 1;
    std::vector<double> b2(3 * (size_t)n, 0.0);
    double spl[MG_MAX_ORDER];
    int z;
    mg_host_bspline(order, 0.0, &z, spl, nullptr);
    for (int d = 0; d < 3; ++d) {
        for (int m = 0; m < n; ++m) {
            if ((order % 2 == 1) && (2 * m == n)) continue;
            // the reference forms cmplx(0, 2 pi m k / n) without a kind, i.e.
            // a single-precision complex: the phase is rounded to float and its
            // exponential evaluated in float (correctly rounded here)
            double re = 0.0, im = 0.0;
            for (int k = 0; k <= order - 2; ++k) {
                float th = (float)(2.0 * kPi * m * k / n);
                float cr = (float)std::cos((double)th), ci = (float)std::sin((double)th);
                re = re + spl[k + 1] * (double)cr;
                im = im + spl[k + 1] * (double)ci;
            }
            b2[d * (size_t)n + m] = 1.0 / (re * re + im * im);
        }
    }
    (void)boxlen;
    size_t n3 = (size_t)nh * nh * nh;
    mf.assign(n3, 0.0);
    ew.assign(n3, 0.0);
    vw.assign(n3, 0.0);
    double fac0 = 4.0 * kPi / vol;
    double expf = -1.0 / (4.0 * (ualpha * ualpha));
    for (int fz = 0; fz < nh; ++fz)
        for (int fy = 0; fy < nh; ++fy)
            for (int kx = 0; kx < nh; ++kx) {
                size_t id = ((size_t)fz * nh + fy) * nh + kx;
                if (kx == 0 && fy == 0 && fz == 0) continue;
                double m2 = sq(kx * TwoPiBoxi[0]) + sq(fy * TwoPiBoxi[1]) + sq(fz * TwoPiBoxi[2]);
                double c = std::exp(m2 * expf) / m2;
                double f = fac0 * c * b2[kx] * b2[n + fy] * b2[2 * (size_t)n + fz];
                mf[id] = f;
                double scale = 1.0;
                if (kx == (n - kx) % n) f = f / 2;
                if (fy == (n - fy) % n) { f = f / 2; scale *= 2.0; }
                if (fz == (n - fz) % n) { f = f / 2; scale *= 2.0; }
                double v = (1.0 + 2 * m2 * expf) * f;
                ew[id] = f * scale;
                vw[id] = v * scale;
            }
}

// k-vectors of the first octant with n^2 <= ncut2, origin excluded, in the
// reference's kn order (nz, ny, nx loops; energy.F90:6765-6782)
void mg_host_kvectors(int ncut, int ncut2, const double TwoPiBoxi[3], double vol, double ualpha,
                      std::vector<int> &kv, std::vector<double> &kfac) {
    kv.clear();
    kfac.clear();
    double fac0 = 2.0 * kPi / vol;
    for (int nz = 0; nz <= ncut; ++nz) {
        double fz = (nz == 0) ? 1.0 : 2.0;
        for (int ny = 0; ny <= ncut; ++ny) {
            double fy = (ny == 0) ? 0.5 : 1.0;
            for (int nx = 0; nx <= ncut; ++nx) {
                if (nx * nx + ny * ny + nz * nz > ncut2) continue;
                if (nx == 0 && ny == 0 && nz == 0) continue;
                double fx = (nx == 0) ? 0.5 : 1.0;
                double k2 = sq(nx * TwoPiBoxi[0]) + sq(ny * TwoPiBoxi[1]) + sq(nz * TwoPiBoxi[2]);
                kv.push_back(nx);
                kv.push_back(ny);
                kv.push_back(nz);
                kv.push_back(0);
                kfac.push_back(fac0 * fz * fy * fx * std::exp(-k2 / (4.0 * (ualpha * ualpha))) / k2);
            }
        }
    }
}

extern "C" int mg_pot_twobody_tab(const mg_pot_params *pp, double *ubuf, int32_t nbuf_cap,
                                  int32_t *nbuf_used, int32_t *iubuflow, double *r2umin,
                                  int32_t *nugrid) {
    return mg_host_table(pp, ubuf, nbuf_cap, nbuf_used, iubuflow, r2umin, nugrid);
}

extern "C" int mg_rcut_to_alpha(double uewaldtol, double rcut, double q2sum, double boxlenshort,
                                double epsi_four_pi, double *ualpha) {
    return mg_host_rcut_to_alpha(uewaldtol, rcut, q2sum, boxlenshort, epsi_four_pi, ualpha);
}
