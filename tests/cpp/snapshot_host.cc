// Host build of afmibins_gb300/csrc/snapshot_io.h for the CPU tests: writes a
// snapshot of known contents and reads files back, with C linkage.
#include <cstring>

#include "snapshot_io.h"

extern "C" {
// a 4x3x2 grid (n = 4, channel), 5 markers with a ring of springs, volumes
int afmib_test_snapshot_write(const char* path) {
    const int N = 24, nxz = 8, M = 5;
    static double u[N], v[N], w[N], phi[N], pp0[N], walls[4 * nxz], wallgrad[6 * nxz], X[3 * M], vol[M];
    static int nstart[M + 1], nidx[2 * M];
    for (int i = 0; i < N; ++i) {
        u[i] = 0.5 + i;
        v[i] = -0.25 * i;
        w[i] = 1.0 / (i + 1);
        phi[i] = 1e-3 * i * i;
        pp0[i] = phi[i] - 1.0;
    }
    for (int i = 0; i < 4 * nxz; ++i) walls[i] = 0.01 * i;
    for (int i = 0; i < 6 * nxz; ++i) wallgrad[i] = -0.5 * i;
    for (int k = 0; k < M; ++k) {
        X[3 * k] = 0.1 * k;
        X[3 * k + 1] = 0.2;
        X[3 * k + 2] = 0.3 + 0.01 * k;
        vol[k] = 1.0 + k;
        nstart[k] = 2 * k;
        nidx[2 * k] = (k + M - 1) % M;
        nidx[2 * k + 1] = (k + 1) % M;
    }
    nstart[M] = 2 * M;
    afmib::snap::Writer wr;
    wr.h.nx = 4;
    wr.h.ny = 3;
    wr.h.nz = 2;
    wr.h.n = 4;
    wr.h.bc = 1;
    wr.h.precision = 1;
    wr.h.half = 1;
    wr.h.substeps = 7;
    wr.h.mg_rho = 0.125;
    wr.add("u", afmib::snap::kF64, u, N);
    wr.add("v", afmib::snap::kF64, v, N);
    wr.add("w", afmib::snap::kF64, w, N);
    wr.add("phi", afmib::snap::kF64, phi, N);
    wr.add("phi_prev0", afmib::snap::kF64, pp0, N);
    wr.add("walls", afmib::snap::kF64, walls, 4 * nxz);
    wr.add("wallgrad", afmib::snap::kF64, wallgrad, 6 * nxz);
    wr.add("X", afmib::snap::kF64, X, 3 * M);
    wr.add("nstart", afmib::snap::kI32, nstart, M + 1);
    wr.add("nidx", afmib::snap::kI32, nidx, 2 * M);
    wr.add("vol", afmib::snap::kF64, vol, M);
    return wr.write(path) ? 0 : 1;
}

// 0 and the section count on success, else 1 and the reason in err
int afmib_test_snapshot_read(const char* path, char* err, int errlen, int* nsections, double* sum_u) {
    afmib::snap::Header h{};
    std::map<std::string, afmib::snap::Section> sec;
    const std::string e = afmib::snap::read(path, &h, &sec);
    std::strncpy(err, e.c_str(), errlen - 1);
    err[errlen - 1] = 0;
    *nsections = (int)sec.size();
    double su = 0;
    auto it = sec.find("u");
    if (it != sec.end())
        for (uint64_t i = 0; i < it->second.count(); ++i) su += it->second.f64()[i];
    *sum_u = su;
    return e.empty() ? 0 : 1;
}
}
