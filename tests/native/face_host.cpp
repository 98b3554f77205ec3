// Host build of the face physics and its hand-derived adjoint (adfvm_gb300/csrc/face.cuh) for
// the CPU unit tests: tests/test_face_adjoint.py compares them with torch autograd of the
// oracle. Test infrastructure only; the product runs the same code on the GPU.
#include <cstring>
#include "face.cuh"

using namespace afvm;

static Phys make_phys(const double* ph) {
    Phys P;
    P.gamma = ph[0];
    P.gm1 = ph[0] - 1;
    P.Cp = ph[1];
    P.Cv = ph[1] / ph[0];
    P.rCv = 1. / P.Cv;
    P.kFac = ph[1] / ph[2];
    P.muModel = (int)ph[3];
    P.mu0 = ph[4];
    P.muAs = ph[5];
    P.muTs = ph[6];
    P.riemann = (int)ph[7];
    P.briemann = (int)ph[8];
    P.small = 1e-30;
    finish_phys(P);
    return P;
}

// the 55 face inputs the tests pass, then the derived geometry (face_derived)
static_assert(sizeof(FaceIn<double>) == 59 * sizeof(double), "FaceIn layout");
static_assert(sizeof(FaceBar<double>) == 40 * sizeof(double), "FaceBar layout");

extern "C" void afvm_host_face(int n, int kind, int inviscid, const double* ph, const double* in, double* F) {
    Phys P = make_phys(ph);
    for (int i = 0; i < n; i++) {
        FaceIn<double> fi;
        memcpy(&fi, in + 55 * (size_t)i, 55 * sizeof(double));
        face_derived(fi);
        double maxaF;
        face_flux<double>(P, kind, inviscid != 0, fi, F + 6 * (size_t)i, maxaF);
        F[6 * (size_t)i + 5] = maxaF;
    }
}

extern "C" void afvm_host_face_vjp(int n, int kind, int inviscid, const double* ph, const double* in,
                                   const double* Fb, double* out) {
    Phys P = make_phys(ph);
    for (int i = 0; i < n; i++) {
        FaceIn<double> fi;
        memcpy(&fi, in + 55 * (size_t)i, 55 * sizeof(double));
        face_derived(fi);
        FaceBar<double> b;
        zero_bar(b);
        face_vjp<double>(P, kind, inviscid != 0, fi, Fb + 5 * (size_t)i, b);
        memcpy(out + 40 * (size_t)i, &b, sizeof(b));
    }
}

// the same VJP in FP32 (the lean local tape: the Roe and viscous intermediates re-evaluated)
extern "C" void afvm_host_face_vjp_f32(int n, int kind, int inviscid, const double* ph, const double* in,
                                       const double* Fb, double* out) {
    Phys P = make_phys(ph);
    P.small = 1e-9;
    finish_phys(P);
    for (int i = 0; i < n; i++) {
        FaceIn<float> fi;
        float* f = &fi.UP[0];
        for (int k = 0; k < 55; k++) f[k] = (float)in[55 * (size_t)i + k];
        face_derived(fi);
        float fb[5];
        for (int k = 0; k < 5; k++) fb[k] = (float)Fb[5 * (size_t)i + k];
        FaceBar<float> b;
        zero_bar(b);
        face_vjp<float>(P, kind, inviscid != 0, fi, fb, b);
        const float* bo = &b.UP[0];
        for (int k = 0; k < 40; k++) out[40 * (size_t)i + k] = bo[k];
    }
}

// the VJP with the geometry adjoints too: out holds 55 values per face, the 40 input adjoints
// then N (3), D (3), lw0, lw1, qw0 (3), qw1 (3) and the adjoint of 1/deltas
static_assert(sizeof(GeoBar<double>) == 15 * sizeof(double), "GeoBar layout");
extern "C" void afvm_host_face_vjp_geo(int n, int kind, int inviscid, const double* ph, const double* in,
                                       const double* Fb, double* out) {
    Phys P = make_phys(ph);
    for (int i = 0; i < n; i++) {
        FaceIn<double> fi;
        memcpy(&fi, in + 55 * (size_t)i, 55 * sizeof(double));
        face_derived(fi);
        FaceBar<double> b;
        zero_bar(b);
        GeoBar<double> g;
        zero_geo(g);
        face_vjp<double>(P, kind, inviscid != 0, fi, Fb + 5 * (size_t)i, b, &g);
        memcpy(out + 55 * (size_t)i, &b, sizeof(b));
        memcpy(out + 55 * (size_t)i + 40, &g, sizeof(g));
    }
}

// The gauge-form flux of FP32 records (face_flux<R, true>): `in` holds absolute values; the
// offsets p - gauge[0], T - gauge[1] are taken in double (as the records' are) and then rounded
// to R. F receives the gauge-form flux and the CFL term, in double.
template <typename R>
static void gauge_faces(int n, int kind, int inviscid, const Phys& P, const double* in, double* F) {
    for (int i = 0; i < n; i++) {
        const double* x = in + 55 * (size_t)i;
        double y[55];
        for (int k = 0; k < 55; k++) y[k] = x[k];
        y[3] -= P.gaugeT; y[8] -= P.gaugeT;
        y[4] -= P.gaugeP; y[9] -= P.gaugeP;
        FaceIn<R> fi;
        R* f = &fi.UP[0];
        for (int k = 0; k < 55; k++) f[k] = (R)y[k];
        face_derived(fi);
        R Fo[5], maxaF;
        face_flux<R, true>(P, kind, inviscid != 0, fi, Fo, maxaF);
        for (int k = 0; k < 5; k++) F[6 * (size_t)i + k] = Fo[k];
        F[6 * (size_t)i + 5] = maxaF;
    }
}

extern "C" void afvm_host_face_gauge(int n, int kind, int inviscid, const double* ph, const double* gauge, int f32,
                                     const double* in, double* F) {
    Phys P = make_phys(ph);
    if (f32) P.small = 1e-9;
    P.gaugeP = gauge[0];
    P.gaugeT = gauge[1];
    P.gaugeH = gauge[2];
    finish_phys(P);
    if (f32)
        gauge_faces<float>(n, kind, inviscid, P, in, F);
    else
        gauge_faces<double>(n, kind, inviscid, P, in, F);
}

// the absolute-form flux in FP32 (the form FP32 records had without a gauge)
extern "C" void afvm_host_face_f32(int n, int kind, int inviscid, const double* ph, const double* in, double* F) {
    Phys P = make_phys(ph);
    P.small = 1e-9;
    finish_phys(P);
    for (int i = 0; i < n; i++) {
        FaceIn<float> fi;
        float* f = &fi.UP[0];
        for (int k = 0; k < 55; k++) f[k] = (float)in[55 * (size_t)i + k];
        face_derived(fi);
        float Fo[5], maxaF;
        face_flux<float>(P, kind, inviscid != 0, fi, Fo, maxaF);
        for (int k = 0; k < 5; k++) F[6 * (size_t)i + k] = Fo[k];
        F[6 * (size_t)i + 5] = maxaF;
    }
}
