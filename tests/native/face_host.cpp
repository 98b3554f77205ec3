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

static_assert(sizeof(FaceIn<double>) == 55 * sizeof(double), "FaceIn layout");
static_assert(sizeof(FaceBar<double>) == 40 * sizeof(double), "FaceBar layout");

extern "C" void afvm_host_face(int n, int kind, int inviscid, const double* ph, const double* in, double* F) {
    Phys P = make_phys(ph);
    for (int i = 0; i < n; i++) {
        FaceIn<double> fi;
        memcpy(&fi, in + 55 * (size_t)i, sizeof(fi));
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
        memcpy(&fi, in + 55 * (size_t)i, sizeof(fi));
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
        memcpy(&fi, in + 55 * (size_t)i, sizeof(fi));
        FaceBar<double> b;
        zero_bar(b);
        GeoBar<double> g;
        zero_geo(g);
        face_vjp<double>(P, kind, inviscid != 0, fi, Fb + 5 * (size_t)i, b, &g);
        memcpy(out + 55 * (size_t)i, &b, sizeof(b));
        memcpy(out + 55 * (size_t)i + 40, &g, sizeof(g));
    }
}
