// Host build of the device double-float math (surfaceonlydeformables_gb300/csrc/sod_dd.cuh) for the
// CPU accuracy tests.  Compiled by tests/test_dd_math.py with g++ -O2 -ffp-contract=off.
#include "sod_dd.cuh"

using namespace sod;

extern "C" {
// each input double x is first rounded to a float pair; `xin` returns the exact value used
void dd_exp_eval(const double *x, double *xin, double *out, int n) {
    for (int i = 0; i < n; i++) {
        const dd a = dd_from(x[i]);
        xin[i] = dd_to(a);
        out[i] = dd_to(dd_exp(a));
    }
}
void dd_sincos_eval(const double *x, double *xin, double *s, double *c, int n) {
    for (int i = 0; i < n; i++) {
        const dd a = dd_from(x[i]);
        xin[i] = dd_to(a);
        dd ss, cc;
        dd_sincos(a, ss, cc);
        s[i] = dd_to(ss);
        c[i] = dd_to(cc);
    }
}
void dd_sqrt_eval(const double *x, double *xin, double *out, int n) {
    for (int i = 0; i < n; i++) {
        const dd a = dd_from(x[i]);
        xin[i] = dd_to(a);
        out[i] = dd_to(dd_sqrt(a));
    }
}
void dd_recip_eval(const double *x, double *xin, double *out, int n) {
    for (int i = 0; i < n; i++) {
        const dd a = dd_from(x[i]);
        xin[i] = dd_to(a);
        out[i] = dd_to(dd_recip(a));
    }
}
// z = (re, im) pairs; out = psi(z) computed from the library's own e^-z
void dd_psi_eval(const double *z, double *zin, double *out, int n) {
    for (int i = 0; i < n; i++) {
        const cdd w = cdd{dd_from(z[2 * i]), dd_from(z[2 * i + 1])};
        zin[2 * i] = dd_to(w.x);
        zin[2 * i + 1] = dd_to(w.y);
        const cdd p = cdd_psi(w, cdd_exp_neg(w));
        out[2 * i] = dd_to(p.x);
        out[2 * i + 1] = dd_to(p.y);
    }
}
void dd_cexp_neg_eval(const double *z, double *zin, double *out, int n) {
    for (int i = 0; i < n; i++) {
        const cdd w = cdd{dd_from(z[2 * i]), dd_from(z[2 * i + 1])};
        zin[2 * i] = dd_to(w.x);
        zin[2 * i + 1] = dd_to(w.y);
        const cdd e = cdd_exp_neg(w);
        out[2 * i] = dd_to(e.x);
        out[2 * i + 1] = dd_to(e.y);
    }
}
// products and sums of dd pairs: out = a*b + c
void dd_fma_eval(const double *a, const double *b, const double *c, double *abc, double *out, int n) {
    for (int i = 0; i < n; i++) {
        const dd x = dd_from(a[i]), y = dd_from(b[i]), z = dd_from(c[i]);
        abc[3 * i] = dd_to(x), abc[3 * i + 1] = dd_to(y), abc[3 * i + 2] = dd_to(z);
        out[i] = dd_to(x * y + z);
    }
}
}
