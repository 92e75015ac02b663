// mg_replay — a compiled caller of the C ABI (include/molsim_gb300.h) that
// replays the reference's step sequences the way its Fortran drivers call
// the hot path: VelVer steps (md.F90:252-357), BDStep steps (bd.F90:120-155)
// and single-particle MC passes (MCPass/SPartMove, mc.F90:1470-1753, with
// GetRandomTrialPos :4527-4580, CheckPartBCTM :4810-4858, Metropolis
// :5135-5178, MCUpdate :5203-5236 and NListDriver after each pass).  It
// uses nothing but the ABI: a host code in any language that can call C
// sees the library the same way.
//
//   mg_replay <input> <output>
//
// Both files are sequences of tagged arrays: a 16-byte name (NUL padded),
// a type byte ('i' int32, 'd' float64), an int64 count, then the values
// (little endian).  The input holds the mg_params fields under their own
// names, the positions "ro" and the run: "run_kind" (0 VelVer, 1 BDStep,
// 2 MC passes), "nstep", and per kind "tstep", "massip", "rod", "rodd" /
// "fac1", "fac2", "iseed" / "iseed", "dtran", "beta".  The output holds "ro",
// "uout" (u%tot, u%rec, u%bond, virial of the last UTotal), "forceo" and per
// kind "rod" / "iseed" / "naccept", "du_acc".
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "molsim_gb300.h"

namespace {

struct Array {
    char type = 'd';
    std::vector<int32_t> i;
    std::vector<double> d;
};

using Record = std::map<std::string, Array>;

[[noreturn]] void die(const char *what, const char *detail) {
    std::fprintf(stderr, "mg_replay: %s%s%s\n", what, detail ? ": " : "", detail ? detail : "");
    std::exit(2);
}

Record read_record(const char *path) {
    FILE *f = std::fopen(path, "rb");
    if (!f) die("cannot open input", path);
    Record r;
    char name[17];
    while (std::fread(name, 1, 16, f) == 16) {
        name[16] = 0;
        char type;
        int64_t n;
        if (std::fread(&type, 1, 1, f) != 1 || std::fread(&n, 8, 1, f) != 1 || n < 0) die("truncated input", name);
        Array a;
        a.type = type;
        if (type == 'i') {
            a.i.resize((size_t)n);
            if (n && std::fread(a.i.data(), 4, (size_t)n, f) != (size_t)n) die("truncated array", name);
        } else if (type == 'd') {
            a.d.resize((size_t)n);
            if (n && std::fread(a.d.data(), 8, (size_t)n, f) != (size_t)n) die("truncated array", name);
        } else {
            die("unknown array type", name);
        }
        r[std::string(name)] = std::move(a);
    }
    std::fclose(f);
    return r;
}

void write_array(FILE *f, const char *name, const double *v, size_t n) {
    char nm[16] = {0};
    std::strncpy(nm, name, 16);
    char type = 'd';
    int64_t c = (int64_t)n;
    std::fwrite(nm, 1, 16, f);
    std::fwrite(&type, 1, 1, f);
    std::fwrite(&c, 8, 1, f);
    if (n) std::fwrite(v, 8, n, f);
}

void write_int(FILE *f, const char *name, int32_t v) {
    char nm[16] = {0};
    std::strncpy(nm, name, 16);
    char type = 'i';
    int64_t c = 1;
    std::fwrite(nm, 1, 16, f);
    std::fwrite(&type, 1, 1, f);
    std::fwrite(&c, 8, 1, f);
    std::fwrite(&v, 4, 1, f);
}

const Array &need(const Record &r, const char *name) {
    auto it = r.find(name);
    if (it == r.end()) die("missing input array", name);
    return it->second;
}
const int32_t *ip(const Record &r, const char *name) {
    auto it = r.find(name);
    return it == r.end() || it->second.i.empty() ? nullptr : it->second.i.data();
}
const double *dp(const Record &r, const char *name) {
    auto it = r.find(name);
    return it == r.end() || it->second.d.empty() ? nullptr : it->second.d.data();
}
int32_t iv(const Record &r, const char *name) {
    const Array &a = need(r, name);
    if (a.i.empty()) die("expected an integer", name);
    return a.i[0];
}
double dv(const Record &r, const char *name) {
    const Array &a = need(r, name);
    if (a.d.empty()) die("expected a real", name);
    return a.d[0];
}

void check(mg_handle *h, int st, const char *what) {
    if (st == MG_OK) return;
    char buf[512] = {0};
    mg_last_error(h, buf, sizeof buf);
    std::fprintf(stderr, "mg_replay: %s: %s: %s\n", what, mg_status_string(st), buf);
    std::exit(3);
}

// Random(idum), mollib.F90:2689-2709: Marsaglia's xorshift combined with
// Park-Miller by Schrage's method; the module state lives here.
struct RefRandom {
    int32_t idum, ix = -1, iy = -1;
    double am = 0.0;
    explicit RefRandom(int32_t seed) : idum(seed) {}
    double operator()() {
        const int32_t ia = 16807, im = 2147483647, iq = 127773, ir = 2836;
        if (idum <= 0 || iy < 0) {
            am = (double)(std::nextafter(1.0f, 0.0f) / (float)im);   // nearest(1.0,-1.0)/im, default real
            int32_t a = idum < 0 ? -idum : idum;
            iy = (888889999 ^ a) | 1;
            ix = 777755555 ^ a;
            idum = a + 1;
        }
        uint32_t x = (uint32_t)ix;
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        ix = (int32_t)x;
        int32_t k = iy / iq;
        iy = ia * (iy - k * iq) - ir * k;
        if (iy < 0) iy += im;
        return am * (double)((im & (ix ^ iy)) | 1);
    }
};

// PBC (molaux.F90:104-146, box): d - L*anint(d/L) where |d| > L/2
double pbc(double d, double len, double half, double inv) {
    return std::fabs(d) > half ? d - len * std::round(d * inv) : d;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: mg_replay <input> <output>\n");
        return 1;
    }
    Record in = read_record(argv[1]);
    mg_params p;
    std::memset(&p, 0, sizeof p);
    p.abi_version = MG_ABI_VERSION;
    p.np = iv(in, "np");
    p.npt = iv(in, "npt");
    p.nptpt = iv(in, "nptpt");
    p.iptpn = ip(in, "iptpn");
    p.iptpt = ip(in, "iptpt");
    p.az = dp(in, "az");
    p.nbuf = (int32_t)need(in, "ubuf").d.size();
    p.ubuf = dp(in, "ubuf");
    p.iubuflow = ip(in, "iubuflow");
    p.r2umin = dp(in, "r2umin");
    p.r2atat = dp(in, "r2atat");
    for (int m = 0; m < 3; ++m) p.boxlen[m] = need(in, "boxlen").d.at(m);
    p.rcut = dv(in, "rcut");
    p.drnlist = dv(in, "drnlist");
    p.txintlist = iv(in, "txintlist");
    p.mode = iv(in, "mode");
    p.form = iv(in, "form");
    p.maxnneigh = iv(in, "maxnneigh");
    p.ewald = iv(in, "ewald");
    p.ualpha = dv(in, "ualpha");
    p.ncut = iv(in, "ncut");
    p.ncutregion_cube = iv(in, "ncutregion_cube");
    p.order = iv(in, "order");
    p.nmesh = iv(in, "nmesh");
    p.lsurf = iv(in, "lsurf");
    p.epsi_four_pi = dv(in, "epsi_four_pi");
    p.force_fac = dv(in, "force_fac");
    p.nbond = in.count("bond_ip") ? (int32_t)in["bond_ip"].i.size() : 0;
    p.bond_ip = ip(in, "bond_ip");
    p.bond_jp = ip(in, "bond_jp");
    p.bond_k = dp(in, "bond_k");
    p.bond_eq = dp(in, "bond_eq");
    p.bond_p = ip(in, "bond_p");
    p.nangle = in.count("angle_ip") ? (int32_t)in["angle_ip"].i.size() : 0;
    p.angle_jm = ip(in, "angle_jm");
    p.angle_ip = ip(in, "angle_ip");
    p.angle_jp = ip(in, "angle_jp");
    p.angle_k = dp(in, "angle_k");
    p.angle_eq = dp(in, "angle_eq");
    p.angle_p = ip(in, "angle_p");

    const int np = p.np;
    std::vector<double> ro(need(in, "ro").d), forceo(3 * (size_t)np), uout(4), u_twob((size_t)p.nptpt + 1);
    if ((int)ro.size() != 3 * np) die("ro has the wrong length", nullptr);

    mg_handle *h = nullptr;
    check(h, mg_create(&p, &h), "mg_create");
    check(h, mg_set_positions(h, ro.data()), "mg_set_positions");
    check(h, mg_nlist_set(h), "mg_nlist_set");

    const int kind = iv(in, "run_kind"), nstep = iv(in, "nstep");
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) die("cannot open output", argv[2]);

    if (kind == 0) {   // VelVer
        std::vector<double> rod(need(in, "rod").d), rodd(need(in, "rodd").d);
        check(h, mg_md_setup(h, dv(in, "tstep"), dp(in, "massip"), rod.data(), rodd.data()), "mg_md_setup");
        check(h, mg_md_run(h, nstep, forceo.data(), uout.data(), rod.data(), rodd.data()), "mg_md_run");
        write_array(out, "rod", rod.data(), rod.size());
    } else if (kind == 1) {   // BDStep
        check(h, mg_bd_setup(h, dp(in, "fac1"), dp(in, "fac2"), iv(in, "iseed")), "mg_bd_setup");
        check(h, mg_bd_run(h, nstep, forceo.data(), uout.data()), "mg_bd_run");
        int32_t seed = 0;
        check(h, mg_bd_get_seed(h, &seed), "mg_bd_get_seed");
        write_int(out, "iseed", seed);
    } else if (kind == 2) {   // MC passes of single-particle moves, particles chosen at random
        check(h, mg_utotal(h, forceo.data(), u_twob.data(), uout.data()), "mg_utotal");
        RefRandom rnd(iv(in, "iseed"));
        const double dtran = dv(in, "dtran"), beta = dv(in, "beta");
        double len[3], half[3], inv[3];
        for (int m = 0; m < 3; ++m) {
            len[m] = p.boxlen[m];
            half[m] = 0.5 * len[m];
            inv[m] = 1.0 / len[m];
        }
        std::vector<double> drostep(3 * (size_t)np), du_twob((size_t)p.nptpt + 1);
        int32_t naccept = 0;
        double du_acc = 0.0;
        for (int pass = 0; pass < nstep; ++pass) {
            std::fill(drostep.begin(), drostep.end(), 0.0);
            for (int ipass = 1; ipass <= np; ++ipass) {
                int ipmove = 1 + (int)(np * rnd());
                ipmove = ipmove < 1 ? 1 : (ipmove > np ? np : ipmove);
                double d[3], rt[3];
                for (int m = 0; m < 3; ++m) d[m] = (rnd() - 0.5) * dtran;   // GetRandomTrialPos, cube
                for (int m = 0; m < 3; ++m) rt[m] = pbc(ro[3 * (ipmove - 1) + m] + d[m], len[m], half[m], inv[m]);
                double du_rec = 0.0, du_tot = 0.0;
                int32_t ovl = 0;
                check(h, mg_dutotal(h, 1, &ipmove, rt, du_twob.data(), &du_rec, &du_tot, &ovl), "mg_dutotal");
                bool acc = false;   // Metropolis, weight 1
                if (!ovl) {
                    double dured = du_tot * beta;
                    if (dured > 87.0) acc = false;
                    else if (dured < -87.0) acc = true;
                    else {
                        double fac = std::exp(-dured);
                        acc = fac > 1.0 || fac > rnd();
                    }
                }
                if (acc) {
                    check(h, mg_accept(h), "mg_accept");
                    for (int m = 0; m < 3; ++m) {
                        ro[3 * (ipmove - 1) + m] = rt[m];
                        drostep[3 * (ipmove - 1) + m] += d[m];
                    }
                    du_acc += du_tot;
                    ++naccept;
                }
            }
            int32_t rebuilt = 0;
            check(h, mg_nlist_update(h, drostep.data(), &rebuilt), "mg_nlist_update");
        }
        check(h, mg_utotal(h, forceo.data(), u_twob.data(), uout.data()), "mg_utotal");
        write_int(out, "naccept", naccept);
        write_array(out, "du_acc", &du_acc, 1);
    } else {
        die("run_kind must be 0, 1 or 2", nullptr);
    }
    check(h, mg_get_positions(h, ro.data()), "mg_get_positions");
    write_array(out, "ro", ro.data(), ro.size());
    write_array(out, "uout", uout.data(), uout.size());
    write_array(out, "forceo", forceo.data(), forceo.size());
    std::fclose(out);
    mg_destroy(h);
    return 0;
}
