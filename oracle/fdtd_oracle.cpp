// CPU oracle for the FDTD hot path. TEST INFRASTRUCTURE ONLY: the product never links, imports or
// calls this code; tests, smoke() and the benchmark's CPU-baseline leg use it as the checker.
//
// A restatement, in the reference's own structure, of the single-slab (NUMDEV = 1) setup and time
// step of ravelec/FDTD fdtdrav.h:
//   * per-cell material arrays painted by bricks, then edge-averaged eps/sigma and harmonic-mean
//     mu/sigma_m with the reference's masks (setBrick 1524-1571, setSigmaEpsSigmaMu 1097-1220);
//   * 18 per-edge update coefficients (setCoefficients 1223-1308);
//   * CPML profiles, cpsi = C*delta and C/kappa per face in the order x_n, x_p, y_n, y_p, z_n, z_p
//     (setABCPML 1747-2160);
//   * lumped z-sources then resistors overriding the Ez coefficients (defineSourceZ 1368-1426,
//     defineResistor 1429-1483);
//   * per step calc_e then calc_h: the three main updates with their masks, source injection and
//     pre-CPML sampling, then the six CPML blocks (calc_e 577-915, calc_h 249-573).
// Templated on the real type: float is the FP32 restatement (rounding sequence written out with
// fmaf where the reference's expressions are contracted), double is the FP64 build used as the
// error reference. Compile with -ffp-contract=off so the compiler adds no contractions of its own.
//
// Parity is pinned by golden fixtures produced by the reference's own kernels (tests/golden).

#include <cmath>
#include <cstdint>
#include <chrono>
#include <cstring>
#include <array>
#include <vector>
#include <string>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class R> inline R FMA(R a, R b, R c);
template <> inline float FMA<float>(float a, float b, float c) { return std::fmaf(a, b, c); }
template <> inline double FMA<double>(double a, double b, double c) { return std::fma(a, b, c); }
template <class R> inline R POW(R a, R b);
template <> inline float POW<float>(float a, float b) { return std::pow(a, b); }
template <> inline double POW<double>(double a, double b) { return std::pow(a, b); }
template <class R> inline R EXP(R a);
template <> inline float EXP<float>(float a) { return std::exp(a); }
template <> inline double EXP<double>(double a) { return std::exp(a); }

std::string g_err;

}  // namespace

extern "C" {

// Scenario in index space (mirrors fdtd_api.h): material index per cell + table, lumped edges,
// point probes. Profiles may be overridden (e.g. with the reference's own) to isolate the update.
typedef struct {
    int nx, ny, nz;
    int pml[6];  // x_n, x_p, y_n, y_p, z_n, z_p
    float dx, dy, dz, dt, eps0, mu0, pi;
    const uint8_t* mat;       // (nz, ny, nx)
    const float* table;       // (n_mat, 3, 4): per axis x, y, z: eps_r, sigma_e, mu_r, sigma_m
    int n_mat;
    int nsrc; const int* src_box; const float* src_r;  // box is,js,ks,ie,je,ke
    int nres; const int* res_box; const float* res_r;
    int nprobe; const int* probe;                       // (nprobe, 4): comp, i, j, k
    // optional 1-D profile override: 18 arrays, per axis x, y, z: b_e, a_e, b_m, a_m, kappa_e,
    // kappa_m (length n_axis); NULL entries keep the oracle's own values
    const float* const* profile_override;
    // optional design region: cells [d0,d3) x [d1,d4) x [d2,d5) take eps_r from design_eps
    // ((d5-d2), (d4-d1), (d3-d0) array, x fastest) instead of the material table
    int design_box[6];
    const double* design_eps;
    // zero-thickness plates, applied in order: (nplate, 7) ints axis, is, js, ks, ie, je, ke and
    // (nplate, 2) floats sigma_e of the two tangential components in axis order
    int nplate; const int* plate; const float* plate_sig;
    // x-directed elements of defineSourceX: boxes is,js,ks,ie,je,ke and resistances
    int nsrcx; const int* srcx_box; const float* srcx_r;
} or_scenario;

const char* or_error(void) { return g_err.c_str(); }

}  // extern "C"

namespace {

template <class R>
struct Sim {
    int NX, NY, NZ;
    int pxn, pxp, pyn, pyp, pzn, pzp;
    R dx, dy, dz, dt, eps0, mu0, pi;
    size_t N;
    // fields
    std::vector<R> Ex, Ey, Ez, Hx, Hy, Hz;
    // coefficients
    std::vector<R> Cexe, Cexhz, Cexhy, Ceye, Ceyhx, Ceyhz, Ceze, Cezhy, Cezhx, Cezj;
    std::vector<R> Chxh, Chxey, Chxez, Chyh, Chyez, Chyex, Chzh, Chzex, Chzey;
    // averaged material
    std::vector<R> eps_x, eps_y, eps_z, sig_x, sig_y, sig_z, mu_x, mu_y, mu_z, sm_x, sm_y, sm_z;
    // psi and cpsi (full volume, as the reference)
    std::vector<R> Psi_eyx, Psi_ezx, Psi_hyx, Psi_hzx, cpsi_eyx, cpsi_ezx, cpsi_hyx, cpsi_hzx;
    std::vector<R> Psi_exy, Psi_ezy, Psi_hxy, Psi_hzy, cpsi_exy, cpsi_ezy, cpsi_hxy, cpsi_hzy;
    std::vector<R> Psi_exz, Psi_eyz, Psi_hxz, Psi_hyz, cpsi_exz, cpsi_eyz, cpsi_hxz, cpsi_hyz;
    // 1-D profiles
    std::vector<R> b_ex, a_ex, b_mx, a_mx, b_ey, a_ey, b_my, a_my, b_ez, a_ez, b_mz, a_mz;
    // lumped sources: boxes, signals (per node) by source
    std::vector<std::array<int, 6>> sbox;
    std::vector<std::vector<R>> signal;
    // probes
    std::vector<std::array<int, 4>> probes;

    inline size_t id(int i, int j, int k) const { return (size_t)i + (size_t)j * NX + (size_t)k * NX * NY; }
};

#define VEC_LIST(X) X(Ex) X(Ey) X(Ez) X(Hx) X(Hy) X(Hz) \
    X(Cexe) X(Cexhz) X(Cexhy) X(Ceye) X(Ceyhx) X(Ceyhz) X(Ceze) X(Cezhy) X(Cezhx) X(Cezj) \
    X(Chxh) X(Chxey) X(Chxez) X(Chyh) X(Chyez) X(Chyex) X(Chzh) X(Chzex) X(Chzey) \
    X(Psi_eyx) X(Psi_ezx) X(Psi_hyx) X(Psi_hzx) X(cpsi_eyx) X(cpsi_ezx) X(cpsi_hyx) X(cpsi_hzx) \
    X(Psi_exy) X(Psi_ezy) X(Psi_hxy) X(Psi_hzy) X(cpsi_exy) X(cpsi_ezy) X(cpsi_hxy) X(cpsi_hzy) \
    X(Psi_exz) X(Psi_eyz) X(Psi_hxz) X(Psi_hyz) X(cpsi_exz) X(cpsi_eyz) X(cpsi_hxz) X(cpsi_hyz)

// setCoefficients form (fdtdrav.h:1250-1303)
template <class R>
inline void coef(R rel, R cond, R dt, R c0, R dplus, R dminus, R& a, R& bp, R& bm) {
    R two_r = (R)2 * rel;
    R dts = dt * cond;
    R num = FMA<R>(two_r, c0, -dts);
    R den = FMA<R>(two_r, c0, dts);
    a = num / den;
    bp = ((R)2 * dt) / (den * dplus);
    bm = ((R)-2 * dt) / (den * dminus);
}

// One face profile of setABCPML (fdtdrav.h:1863-1891 and its mirrors): rho is the double
// expression of the reference rounded to R.
template <class R>
inline void profile(R roe, R rom, R delta, R dt, R eps0, R mu0, R pi,
                    R& be, R& ae, R& bm, R& am, R& ke, R& km) {
    const R npml = 3, sigma_factor = (R)1.5, kappa_max = 5, alpha_max = (R)0.05, alpha_min = (R)0.00;
    R sigma_opt = (npml + 1) / ((R)150 * pi * (R)1 * delta);
    R sigma_max = sigma_factor * sigma_opt;
    R sigma_pe = sigma_max * POW<R>(roe, npml);
    R sigma_pm = sigma_max * POW<R>(rom, npml);
    sigma_pm = sigma_pm * (mu0 / eps0);
    R kappa_e = FMA<R>(kappa_max - 1, POW<R>(roe, npml), (R)1);
    R kappa_m = FMA<R>(kappa_max - 1, POW<R>(rom, npml), (R)1);
    R alpha_e = FMA<R>(alpha_max - alpha_min, (R)1 - roe, alpha_min);
    R alpha_m = FMA<R>(alpha_max - alpha_min, (R)1 - rom, alpha_min);
    alpha_m = alpha_m * (mu0 / eps0);
    be = EXP<R>((-dt / eps0) * ((sigma_pe / kappa_e) + alpha_e));
    ae = ((R)1 / delta) * (be - 1) * sigma_pe / (kappa_e * FMA<R>(kappa_e, alpha_e, sigma_pe));
    bm = EXP<R>((-dt / mu0) * ((sigma_pm / kappa_m) + alpha_m));
    am = ((R)1 / delta) * (bm - 1) * sigma_pm / (kappa_m * FMA<R>(kappa_m, alpha_m, sigma_pm));
    ke = kappa_e;
    km = kappa_m;
}

template <class R>
int setup(Sim<R>& s, const or_scenario* sc, const float* signal_per_node, int n_sig) {
    s.NX = sc->nx; s.NY = sc->ny; s.NZ = sc->nz;
    s.pxn = sc->pml[0]; s.pxp = sc->pml[1]; s.pyn = sc->pml[2]; s.pyp = sc->pml[3]; s.pzn = sc->pml[4]; s.pzp = sc->pml[5];
    s.dx = sc->dx; s.dy = sc->dy; s.dz = sc->dz; s.dt = sc->dt; s.eps0 = sc->eps0; s.mu0 = sc->mu0; s.pi = sc->pi;
    s.N = (size_t)s.NX * s.NY * s.NZ;
    const R tiny = (R)1.2e-38f;
    const size_t N = s.N;
#define ALLOC(v) s.v.assign(N, tiny);
    VEC_LIST(ALLOC)
#undef ALLOC
    const int NX = s.NX, NY = s.NY, NZ = s.NZ;
    // per-cell material of each axis (setBrick, fdtdrav.h:1524-1571) and the edge averages of each
    // component over its own axis' values (setSigmaEpsSigmaMu, fdtdrav.h:1097-1220), init 1 / 1.2e-38
    std::vector<R> ceps[3], csig[3], cmu[3], csm[3];
    for (int a = 0; a < 3; ++a) {
        ceps[a].resize(N); csig[a].resize(N); cmu[a].resize(N); csm[a].resize(N);
        for (size_t n = 0; n < N; ++n) {
            const float* t = sc->table + 12 * sc->mat[n] + 4 * a;
            ceps[a][n] = t[0]; csig[a][n] = t[1]; cmu[a][n] = t[2]; csm[a][n] = t[3];
        }
    }
    if (sc->design_eps) {
        const int* d = sc->design_box;
        for (int k = d[2]; k < d[5]; ++k)
            for (int j = d[1]; j < d[4]; ++j)
                for (int i = d[0]; i < d[3]; ++i)
                    for (int a = 0; a < 3; ++a)
                        ceps[a][s.id(i, j, k)] =
                            (R)sc->design_eps[((size_t)(k - d[2]) * (d[4] - d[1]) + (j - d[1])) * (d[3] - d[0]) + (i - d[0])];
    }
    s.eps_x.assign(N, 1); s.eps_y.assign(N, 1); s.eps_z.assign(N, 1);
    s.mu_x.assign(N, 1); s.mu_y.assign(N, 1); s.mu_z.assign(N, 1);
    s.sig_x.assign(N, tiny); s.sig_y.assign(N, tiny); s.sig_z.assign(N, tiny);
    s.sm_x.assign(N, tiny); s.sm_y.assign(N, tiny); s.sm_z.assign(N, tiny);
    auto avg4 = [](R a, R b, R c, R d) { return (((a + b) + c) + d) * (R)0.25; };
    auto harm = [](R a, R b) { return ((R)2 * a * b) / (a + b); };
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                size_t n = s.id(i, j, k);
                if (j > 0 && k > 0) {
                    const std::vector<R>&e = ceps[0], &g = csig[0];
                    size_t a = n, b = s.id(i, j - 1, k), c = s.id(i, j, k - 1), d = s.id(i, j - 1, k - 1);
                    s.eps_x[n] = avg4(e[a], e[b], e[c], e[d]);
                    s.sig_x[n] = avg4(g[a], g[b], g[c], g[d]);
                }
                if (i > 0 && k > 0) {
                    const std::vector<R>&e = ceps[1], &g = csig[1];
                    size_t a = n, b = s.id(i - 1, j, k), c = s.id(i, j, k - 1), d = s.id(i - 1, j, k - 1);
                    s.eps_y[n] = avg4(e[a], e[b], e[c], e[d]);
                    s.sig_y[n] = avg4(g[a], g[b], g[c], g[d]);
                }
                if (i > 0 && j > 0) {
                    const std::vector<R>&e = ceps[2], &g = csig[2];
                    size_t a = n, b = s.id(i - 1, j, k), c = s.id(i, j - 1, k), d = s.id(i - 1, j - 1, k);
                    s.eps_z[n] = avg4(e[a], e[b], e[c], e[d]);
                    s.sig_z[n] = avg4(g[a], g[b], g[c], g[d]);
                }
                if (i > 0) { size_t b = s.id(i - 1, j, k); s.mu_x[n] = harm(cmu[0][n], cmu[0][b]); s.sm_x[n] = harm(csm[0][n], csm[0][b]); }
                if (j > 0) { size_t b = s.id(i, j - 1, k); s.mu_y[n] = harm(cmu[1][n], cmu[1][b]); s.sm_y[n] = harm(csm[1][n], csm[1][b]); }
                if (k > 0) { size_t b = s.id(i, j, k - 1); s.mu_z[n] = harm(cmu[2][n], cmu[2][b]); s.sm_z[n] = harm(csm[2][n], csm[2][b]); }
            }
    // definePlateX / Y / Z (fdtdrav.h:1574-1679, applied between the averages and setCoefficients,
    // fdtdrav.h:4162-4182): each plate sets sigma_e of the edges its kernel's conditions select
    for (int q = 0; q < sc->nplate; ++q) {
        const int* pl = sc->plate + 7 * q;
        const int axis = pl[0], is = pl[1], js = pl[2], ks = pl[3], ie = pl[4], je = pl[5], ke = pl[6];
        const R sa = (R)sc->plate_sig[2 * q], sb = (R)sc->plate_sig[2 * q + 1];
        for (int k = 0; k < NZ; ++k)
            for (int j = 0; j < NY; ++j)
                for (int i = 0; i < NX; ++i) {
                    const size_t n = s.id(i, j, k);
                    if (axis == 0) {
                        if (i == is && j >= js && j < je && k >= ks && k <= ke) s.sig_y[n] = sa;
                        if (i == is && j >= js && j <= je && k >= ks && k < ke) s.sig_z[n] = sb;
                    } else if (axis == 1) {
                        if (i >= is && i <= ie && j == js && k >= ks && k < ke) s.sig_z[n] = sb;
                        if (i >= is && i < ie && j == js && k >= ks && k <= ke) s.sig_x[n] = sa;
                    } else {
                        if (i >= is && i < ie && j >= js && j <= je && k == ks) s.sig_x[n] = sa;
                        if (i >= is && i <= ie && j >= js && j < je && k == ks) s.sig_y[n] = sb;
                    }
                }
    }
    // setCoefficients with its masks
    const R dt = s.dt, dx = s.dx, dy = s.dy, dz = s.dz;
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                size_t n = s.id(i, j, k);
                if (i < NX && j < NY - 1 && k < NZ - 1) coef<R>(s.mu_x[n], s.sm_x[n], dt, s.mu0, dz, dy, s.Chxh[n], s.Chxey[n], s.Chxez[n]);
                if (i < NX - 1 && j < NY && k < NZ - 1) coef<R>(s.mu_y[n], s.sm_y[n], dt, s.mu0, dx, dz, s.Chyh[n], s.Chyez[n], s.Chyex[n]);
                if (i < NX - 1 && j < NY - 1 && k < NZ) coef<R>(s.mu_z[n], s.sm_z[n], dt, s.mu0, dy, dx, s.Chzh[n], s.Chzex[n], s.Chzey[n]);
                if (i < NX - 1 && j < NY - 1 && k < NZ - 1 && j > 0 && k > 0) coef<R>(s.eps_x[n], s.sig_x[n], dt, s.eps0, dy, dz, s.Cexe[n], s.Cexhz[n], s.Cexhy[n]);
                if (i < NX - 1 && j < NY - 1 && k < NZ - 1 && i > 0 && k > 0) coef<R>(s.eps_y[n], s.sig_y[n], dt, s.eps0, dz, dx, s.Ceye[n], s.Ceyhx[n], s.Ceyhz[n]);
                if (i < NX - 1 && j < NY - 1 && k < NZ - 1 && i > 0 && j > 0) coef<R>(s.eps_z[n], s.sig_z[n], dt, s.eps0, dx, dy, s.Ceze[n], s.Cezhy[n], s.Cezhx[n]);
            }
    // setABCPML: 1-D profiles then per-face cpsi and kappa division
    auto line = [&](std::vector<R>& v, int n) { v.assign((size_t)n, tiny); };
    line(s.b_ex, NX); line(s.a_ex, NX); line(s.b_mx, NX); line(s.a_mx, NX);
    line(s.b_ey, NY); line(s.a_ey, NY); line(s.b_my, NY); line(s.a_my, NY);
    line(s.b_ez, NZ); line(s.a_ez, NZ); line(s.b_mz, NZ); line(s.a_mz, NZ);
    std::vector<R> ke_x(NX, 1), km_x(NX, 1), ke_y(NY, 1), km_y(NY, 1), ke_z(NZ, 1), km_z(NZ, 1);
    auto axis_profile = [&](int n_nodes, int pn, int pp, R delta, std::vector<R>& be, std::vector<R>& ae,
                            std::vector<R>& bm, std::vector<R>& am, std::vector<R>& ke, std::vector<R>& km) {
        for (int q = 0; q < n_nodes; ++q) {
            double roe, rom;
            bool in = false;
            if (q < pn) {  // n face: (P - q - 0.75)/P in double (fdtdrav.h:1863-1864)
                float a = (float)pn - (float)q;
                roe = ((double)a - 0.75) / (double)(float)pn; rom = ((double)a - 0.25) / (double)(float)pn; in = true;
            }
            if (q >= n_nodes - pp) {  // p face: (q - (N - P - 1) - 0.75)/P (fdtdrav.h:1916-1917)
                float a = (float)q - (((float)n_nodes - (float)pp) - 1.0f);
                roe = ((double)a - 0.75) / (double)(float)pp; rom = ((double)a - 0.25) / (double)(float)pp; in = true;
            }
            if (!in) continue;
            profile<R>((R)(float)roe, (R)(float)rom, delta, s.dt, s.eps0, s.mu0, s.pi, be[q], ae[q], bm[q], am[q], ke[q], km[q]);
        }
    };
    axis_profile(NX, s.pxn, s.pxp, dx, s.b_ex, s.a_ex, s.b_mx, s.a_mx, ke_x, km_x);
    axis_profile(NY, s.pyn, s.pyp, dy, s.b_ey, s.a_ey, s.b_my, s.a_my, ke_y, km_y);
    axis_profile(NZ, s.pzn, s.pzp, dz, s.b_ez, s.a_ez, s.b_mz, s.a_mz, ke_z, km_z);
    if (sc->profile_override) {
        std::vector<R>* dst[18] = {&s.b_ex, &s.a_ex, &s.b_mx, &s.a_mx, &ke_x, &km_x, &s.b_ey, &s.a_ey, &s.b_my, &s.a_my,
                                   &ke_y, &km_y, &s.b_ez, &s.a_ez, &s.b_mz, &s.a_mz, &ke_z, &km_z};
        for (int q = 0; q < 18; ++q)
            if (sc->profile_override[q])
                for (size_t t = 0; t < dst[q]->size(); ++t) (*dst[q])[t] = (R)sc->profile_override[q][t];
    }
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                size_t n = s.id(i, j, k);
                if (i < s.pxn || i >= NX - s.pxp) {
                    s.cpsi_eyx[n] = s.Ceyhz[n] * dx; s.cpsi_ezx[n] = s.Cezhy[n] * dx;
                    s.cpsi_hyx[n] = s.Chyez[n] * dx; s.cpsi_hzx[n] = s.Chzey[n] * dx;
                    s.Ceyhz[n] = s.Ceyhz[n] / ke_x[i]; s.Cezhy[n] = s.Cezhy[n] / ke_x[i];
                    s.Chyez[n] = s.Chyez[n] / km_x[i]; s.Chzey[n] = s.Chzey[n] / km_x[i];
                }
                if (j < s.pyn || j >= NY - s.pyp) {
                    s.cpsi_exy[n] = s.Cexhz[n] * dy; s.cpsi_ezy[n] = s.Cezhx[n] * dy;
                    s.cpsi_hxy[n] = s.Chxez[n] * dy; s.cpsi_hzy[n] = s.Chzex[n] * dy;
                    s.Cexhz[n] = s.Cexhz[n] / ke_y[j]; s.Cezhx[n] = s.Cezhx[n] / ke_y[j];
                    s.Chxez[n] = s.Chxez[n] / km_y[j]; s.Chzex[n] = s.Chzex[n] / km_y[j];
                }
                if (k < s.pzn || k >= NZ - s.pzp) {
                    s.cpsi_exz[n] = s.Cexhy[n] * dz; s.cpsi_eyz[n] = s.Ceyhx[n] * dz;
                    s.cpsi_hxz[n] = s.Chxey[n] * dz; s.cpsi_hyz[n] = s.Chyex[n] * dz;
                    s.Cexhy[n] = s.Cexhy[n] / ke_z[k]; s.Ceyhx[n] = s.Ceyhx[n] / ke_z[k];
                    s.Chxey[n] = s.Chxey[n] / km_z[k]; s.Chyex[n] = s.Chyex[n] / km_z[k];
                }
            }
    // defineSourceZ / defineResistor (fdtdrav.h:1368-1483)
    auto lumped = [&](const int* bx, float rs_f, bool is_source) {
        R is = bx[0], js = bx[1], ks = bx[2], ie = bx[3], je = bx[4], ke = bx[5];
        R r_comp = (((R)1 + ie) - is) * (((R)1 + je) - js) / (ke - ks);
        r_comp = r_comp * (R)rs_f;
        R rfactor = (dt * dz) / ((r_comp * dx) * dy);
        R rfactor_aux = (r_comp * dx) * dy;
        for (int k = bx[2]; k < bx[5]; ++k)
            for (int j = bx[1]; j <= bx[4]; ++j)
                for (int i = bx[0]; i <= bx[3]; ++i) {
                    size_t n = s.id(i, j, k);
                    R two_e = (R)2 * s.eps_z[n];
                    R dts = dt * s.sig_z[n];
                    R den = FMA<R>(two_e, s.eps0, dts) + rfactor;
                    R num = FMA<R>(two_e, s.eps0, -dts) - rfactor;
                    s.Ceze[n] = num / den;
                    s.Cezhy[n] = (((R)2 * dt) / dx) / den;
                    s.Cezhx[n] = (((R)-2 * dt) / dy) / den;
                    if (is_source) s.Cezj[n] = (((R)-2 * dt) / rfactor_aux) / den;
                }
    };
    for (int q = 0; q < sc->nsrc; ++q) {
        lumped(sc->src_box + 6 * q, sc->src_r[q], true);
        std::array<int, 6> b;
        for (int t = 0; t < 6; ++t) b[t] = sc->src_box[6 * q + t];
        s.sbox.push_back(b);
        std::vector<R> sig((size_t)n_sig);
        for (int m = 0; m < n_sig; ++m) sig[m] = (R)signal_per_node[(size_t)q * n_sig + m];
        s.signal.push_back(sig);
    }
    for (int q = 0; q < sc->nres; ++q) lumped(sc->res_box + 6 * q, sc->res_r[q], false);
    // defineSourceX (fdtdrav.h:1311-1365): Ex edges i in [is,ie), j in [js,ie] (its j bound),
    // k in [ks,ke]; Cexj is never used (calc_e leaves the x injection out, fdtdrav.h:681)
    for (int q = 0; q < sc->nsrcx; ++q) {
        const int* bx = sc->srcx_box + 6 * q;
        R is = bx[0], js = bx[1], ks = bx[2], ie = bx[3], je = bx[4], ke = bx[5];
        R r_comp = (((R)1 + je) - js) * (((R)1 + ke) - ks) / (ie - is);
        r_comp = r_comp * (R)sc->srcx_r[q];
        R rfactor = (dt * dx) / ((r_comp * dz) * dy);
        for (int k = bx[2]; k <= bx[5]; ++k)
            for (int j = bx[1]; j <= bx[3]; ++j)
                for (int i = bx[0]; i < bx[3]; ++i) {
                    size_t n = s.id(i, j, k);
                    R two_e = (R)2 * s.eps_x[n];
                    R dts = dt * s.sig_x[n];
                    R den = FMA<R>(two_e, s.eps0, dts) + rfactor;
                    R num = FMA<R>(two_e, s.eps0, -dts) - rfactor;
                    s.Cexe[n] = num / den;
                    s.Cexhz[n] = (((R)2 * dt) / dy) / den;
                    s.Cexhy[n] = (((R)-2 * dt) / dz) / den;
                }
    }
    for (int p = 0; p < sc->nprobe; ++p) {
        std::array<int, 4> pr;
        for (int t = 0; t < 4; ++t) pr[t] = sc->probe[4 * p + t];
        s.probes.push_back(pr);
    }
    return 0;
}

// calc_e (fdtdrav.h:577-915) for all nodes; samples E probes into `row`.
template <class R>
void calc_e(Sim<R>& s, int m, R* row) {
    const int NX = s.NX, NY = s.NY, NZ = s.NZ;
    const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const size_t n = s.id(i, j, k);
                if (i < NX - 1 && j < NY - 1 && k < NZ - 1 && j > 0 && k > 0)
                    s.Ex[n] = FMA<R>(s.Cexhy[n], s.Hy[n] - s.Hy[n - sz], FMA<R>(s.Cexe[n], s.Ex[n], s.Cexhz[n] * (s.Hz[n] - s.Hz[n - sy])));
                if (i < NX - 1 && j < NY - 1 && k < NZ - 1 && k > 0 && i > 0)
                    s.Ey[n] = FMA<R>(s.Ceyhz[n], s.Hz[n] - s.Hz[n - sx], FMA<R>(s.Ceye[n], s.Ey[n], s.Ceyhx[n] * (s.Hx[n] - s.Hx[n - sz])));
                if (i < NX - 1 && j < NY - 1 && k < NZ - 1 && j > 0 && i > 0) {
                    R v = FMA<R>(s.Cezhx[n], s.Hx[n] - s.Hx[n - sy], FMA<R>(s.Ceze[n], s.Ez[n], s.Cezhy[n] * (s.Hy[n] - s.Hy[n - sx])));
                    for (size_t q = 0; q < s.sbox.size(); ++q) {
                        const auto& b = s.sbox[q];
                        if (i >= b[0] && i <= b[3] && j >= b[1] && j <= b[4] && k >= b[2] && k < b[5]) {
                            R sig = m < (int)s.signal[q].size() ? s.signal[q][m] : (R)0;
                            v = FMA<R>(s.Cezj[n], sig, v);
                        }
                    }
                    s.Ez[n] = v;
                }
                // pre-CPML samples
                for (size_t p = 0; p < s.probes.size(); ++p) {
                    const auto& pr = s.probes[p];
                    if (pr[0] < 3 && pr[1] == i && pr[2] == j && pr[3] == k)
                        row[p] = pr[0] == 0 ? s.Ex[n] : pr[0] == 1 ? s.Ey[n] : s.Ez[n];
                }
                // CPML x_n and x_p
                if (((i > 0 && i < s.pxn) || (i > NX - s.pxp - 1 && i < NX - 1)) && j < NY - 1 && k < NZ - 1) {
                    s.Psi_eyx[n] = FMA<R>(s.b_ex[i], s.Psi_eyx[n], s.a_ex[i] * (s.Hz[n] - s.Hz[n - sx]));
                    s.Psi_ezx[n] = FMA<R>(s.b_ex[i], s.Psi_ezx[n], s.a_ex[i] * (s.Hy[n] - s.Hy[n - sx]));
                    if (k > 0) s.Ey[n] = FMA<R>(s.cpsi_eyx[n], s.Psi_eyx[n], s.Ey[n]);
                    if (j > 0) s.Ez[n] = FMA<R>(s.cpsi_ezx[n], s.Psi_ezx[n], s.Ez[n]);
                }
                // y_n and y_p
                if (i < NX - 1 && ((j > 0 && j < s.pyn) || (j > NY - s.pyp - 1 && j < NY - 1)) && k < NZ - 1) {
                    s.Psi_exy[n] = FMA<R>(s.b_ey[j], s.Psi_exy[n], s.a_ey[j] * (s.Hz[n] - s.Hz[n - sy]));
                    s.Psi_ezy[n] = FMA<R>(s.b_ey[j], s.Psi_ezy[n], s.a_ey[j] * (s.Hx[n] - s.Hx[n - sy]));
                    if (k > 0) s.Ex[n] = FMA<R>(s.cpsi_exy[n], s.Psi_exy[n], s.Ex[n]);
                    if (i > 0) s.Ez[n] = FMA<R>(s.cpsi_ezy[n], s.Psi_ezy[n], s.Ez[n]);
                }
                // z_n and z_p
                if (i < NX - 1 && j < NY - 1 && ((k > 0 && k < s.pzn) || (k > NZ - s.pzp - 1 && k < NZ - 1))) {
                    s.Psi_exz[n] = FMA<R>(s.b_ez[k], s.Psi_exz[n], s.a_ez[k] * (s.Hy[n] - s.Hy[n - sz]));
                    s.Psi_eyz[n] = FMA<R>(s.b_ez[k], s.Psi_eyz[n], s.a_ez[k] * (s.Hx[n] - s.Hx[n - sz]));
                    if (j > 0) s.Ex[n] = FMA<R>(s.cpsi_exz[n], s.Psi_exz[n], s.Ex[n]);
                    if (i > 0) s.Ey[n] = FMA<R>(s.cpsi_eyz[n], s.Psi_eyz[n], s.Ey[n]);
                }
            }
}

// calc_h (fdtdrav.h:249-573) for all nodes; samples H probes into `row`.
template <class R>
void calc_h(Sim<R>& s, R* row) {
    const int NX = s.NX, NY = s.NY, NZ = s.NZ;
    const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const size_t n = s.id(i, j, k);
                // the reference's Hx statement (fdtdrav.h:338) is contracted with Chxh*Hx as the addend
                if (i < NX && j < NY - 1 && k < NZ - 1)
                    s.Hx[n] = FMA<R>(s.Chxez[n], s.Ez[n + sy] - s.Ez[n], FMA<R>(s.Chxey[n], s.Ey[n + sz] - s.Ey[n], s.Chxh[n] * s.Hx[n]));
                if (i < NX - 1 && j < NY && k < NZ - 1)
                    s.Hy[n] = FMA<R>(s.Chyex[n], s.Ex[n + sz] - s.Ex[n], FMA<R>(s.Chyh[n], s.Hy[n], s.Chyez[n] * (s.Ez[n + sx] - s.Ez[n])));
                if (i < NX - 1 && j < NY - 1 && k < NZ)
                    s.Hz[n] = FMA<R>(s.Chzey[n], s.Ey[n + sx] - s.Ey[n], FMA<R>(s.Chzh[n], s.Hz[n], s.Chzex[n] * (s.Ex[n + sy] - s.Ex[n])));
                for (size_t p = 0; p < s.probes.size(); ++p) {
                    const auto& pr = s.probes[p];
                    if (pr[0] >= 3 && pr[1] == i && pr[2] == j && pr[3] == k)
                        row[p] = pr[0] == 3 ? s.Hx[n] : pr[0] == 4 ? s.Hy[n] : s.Hz[n];
                }
                if (((i < s.pxn) || (i > NX - s.pxp - 1 && i < NX - 1)) && j < NY && k < NZ) {
                    // the psi differences reach one node past the last (i+1); they exist for every node the add masks use
                    if (i + 1 < NX) {
                        s.Psi_hyx[n] = FMA<R>(s.b_mx[i], s.Psi_hyx[n], s.a_mx[i] * (s.Ez[n + sx] - s.Ez[n]));
                        s.Psi_hzx[n] = FMA<R>(s.b_mx[i], s.Psi_hzx[n], s.a_mx[i] * (s.Ey[n + sx] - s.Ey[n]));
                    }
                    if (k < NZ - 1) s.Hy[n] = FMA<R>(s.cpsi_hyx[n], s.Psi_hyx[n], s.Hy[n]);
                    if (j < NY - 1) s.Hz[n] = FMA<R>(s.cpsi_hzx[n], s.Psi_hzx[n], s.Hz[n]);
                }
                if (i < NX && ((j < s.pyn) || (j > NY - s.pyp - 1 && j < NY - 1)) && k < NZ) {
                    if (j + 1 < NY) {
                        s.Psi_hxy[n] = FMA<R>(s.b_my[j], s.Psi_hxy[n], s.a_my[j] * (s.Ez[n + sy] - s.Ez[n]));
                        s.Psi_hzy[n] = FMA<R>(s.b_my[j], s.Psi_hzy[n], s.a_my[j] * (s.Ex[n + sy] - s.Ex[n]));
                    }
                    if (k < NZ - 1) s.Hx[n] = FMA<R>(s.cpsi_hxy[n], s.Psi_hxy[n], s.Hx[n]);
                    if (i < NX - 1) s.Hz[n] = FMA<R>(s.cpsi_hzy[n], s.Psi_hzy[n], s.Hz[n]);
                }
                if (i < NX && j < NY && ((k < s.pzn) || (k > NZ - s.pzp - 1 && k < NZ - 1))) {
                    if (k + 1 < NZ) {
                        s.Psi_hxz[n] = FMA<R>(s.b_mz[k], s.Psi_hxz[n], s.a_mz[k] * (s.Ey[n + sz] - s.Ey[n]));
                        // the reference's Psi_hyz statement (fdtdrav.h:537) is contracted with b*psi as the addend
                        s.Psi_hyz[n] = FMA<R>(s.a_mz[k], s.Ex[n + sz] - s.Ex[n], s.b_mz[k] * s.Psi_hyz[n]);
                    }
                    if (j < NY - 1) s.Hx[n] = FMA<R>(s.cpsi_hxz[n], s.Psi_hxz[n], s.Hx[n]);
                    if (i < NX - 1) s.Hy[n] = FMA<R>(s.cpsi_hyz[n], s.Psi_hyz[n], s.Hy[n]);
                }
            }
}

template <class R>
std::vector<R>* field(Sim<R>& s, int c) {
    std::vector<R>* f[6] = {&s.Ex, &s.Ey, &s.Ez, &s.Hx, &s.Hy, &s.Hz};
    return f[c];
}

// The 12 psi arrays in the reference's order: E x, y, z faces then H x, y, z faces.
template <class R>
std::vector<R>* psi_arr(Sim<R>& s, int q) {
    std::vector<R>* a[12] = {&s.Psi_eyx, &s.Psi_ezx, &s.Psi_exy, &s.Psi_ezy, &s.Psi_exz, &s.Psi_eyz,
                             &s.Psi_hyx, &s.Psi_hzx, &s.Psi_hxy, &s.Psi_hzy, &s.Psi_hxz, &s.Psi_hyz};
    return a[q];
}

// Wall time of the time loop of the last run() (setup and copies excluded), for the CPU baseline.
double g_last_step_seconds = 0.0;

template <class R>
int run(const or_scenario* sc, int steps, const float* signal_per_node, int n_sig,
        const float* init_fields, R* probes_out, R* fields_out, int nthreads, int onestep_m,
        const float* init_psi = nullptr, R* psi_out = nullptr) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    Sim<R> s;
    if (setup<R>(s, sc, signal_per_node, n_sig)) return -1;
    if (init_fields)
        for (int c = 0; c < 6; ++c)
            for (size_t n = 0; n < s.N; ++n) (*field(s, c))[n] = (R)init_fields[(size_t)c * s.N + n];
    if (init_psi)
        for (int q = 0; q < 12; ++q)
            for (size_t n = 0; n < s.N; ++n) (*psi_arr(s, q))[n] = (R)init_psi[(size_t)q * s.N + n];
    const size_t np = s.probes.size();
    std::vector<R> row(np ? np : 1);
    if (onestep_m >= 0) {  // one calc_e then one calc_h at time index onestep_m
        calc_e<R>(s, onestep_m, row.data());
        if (fields_out) for (int c = 0; c < 3; ++c) std::memcpy(fields_out + (size_t)c * s.N, field(s, c)->data(), s.N * sizeof(R));
        calc_h<R>(s, row.data());
        if (fields_out) for (int c = 3; c < 6; ++c) std::memcpy(fields_out + (size_t)c * s.N, field(s, c)->data(), s.N * sizeof(R));
        if (psi_out) for (int q = 0; q < 12; ++q) std::memcpy(psi_out + (size_t)q * s.N, psi_arr(s, q)->data(), s.N * sizeof(R));
        return 0;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (int m = 0; m < steps; ++m) {
        calc_e<R>(s, m, row.data());
        calc_h<R>(s, row.data());
        if (probes_out) for (size_t p = 0; p < np; ++p) probes_out[(size_t)m * np + p] = row[p];
    }
    g_last_step_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (fields_out)
        for (int c = 0; c < 6; ++c) std::memcpy(fields_out + (size_t)c * s.N, field(s, c)->data(), s.N * sizeof(R));
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Discrete adjoint of the update above (the reference has none; this is the checker of the GPU
// adjoint). Figure of merit J = sum_m dt * Ez(p)^2 over the samples of steps m = 0..N-1 at an Ez
// probe outside the CPML. The adjoint state holds dJ/d(field) and dJ/d(psi) at a point of the
// forward sequence; reverse_h undoes calc_h, reverse_e undoes calc_e (transposes of the exact
// linear maps, CPML recurrences and lumped-edge coefficients included).
// ---------------------------------------------------------------------------------------------

template <class R>
struct Adj {
    std::vector<R> ex, ey, ez, hx, hy, hz;
    std::vector<R> psi_eyx, psi_ezx, psi_exy, psi_ezy, psi_exz, psi_eyz;
    std::vector<R> psi_hyx, psi_hzx, psi_hxy, psi_hzy, psi_hxz, psi_hyz;
    explicit Adj(size_t N) {
        for (std::vector<R>* v : {&ex, &ey, &ez, &hx, &hy, &hz, &psi_eyx, &psi_ezx, &psi_exy, &psi_ezy, &psi_exz, &psi_eyz,
                                  &psi_hyx, &psi_hzx, &psi_hxy, &psi_hzy, &psi_hxz, &psi_hyz})
            v->assign(N, (R)0);
    }
};

template <class R>
void reverse_h(const Sim<R>& s, Adj<R>& a) {
    const int NX = s.NX, NY = s.NY, NZ = s.NZ;
    const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const size_t n = s.id(i, j, k);
                const bool xs = (i < s.pxn) || (i > NX - s.pxp - 1 && i < NX - 1);
                const bool ys = (j < s.pyn) || (j > NY - s.pyp - 1 && j < NY - 1);
                const bool zs = (k < s.pzn) || (k > NZ - s.pzp - 1 && k < NZ - 1);
                if (j < NY - 1 && k < NZ - 1) {  // Hx
                    const R L = a.hx[n];
                    const R my = ys ? a.psi_hxy[n] + s.cpsi_hxy[n] * L : 0;
                    const R mz = zs ? a.psi_hxz[n] + s.cpsi_hxz[n] * L : 0;
                    if (ys) a.psi_hxy[n] = s.b_my[j] * my;
                    if (zs) a.psi_hxz[n] = s.b_mz[k] * mz;
                    const R gy = s.Chxey[n] * L + (zs ? s.a_mz[k] * mz : 0);
                    const R gz = s.Chxez[n] * L + (ys ? s.a_my[j] * my : 0);
                    a.ey[n + sz] += gy; a.ey[n] -= gy;
                    a.ez[n + sy] += gz; a.ez[n] -= gz;
                    a.hx[n] = s.Chxh[n] * L;
                }
                if (i < NX - 1 && k < NZ - 1) {  // Hy
                    const R L = a.hy[n];
                    const R mx = xs ? a.psi_hyx[n] + s.cpsi_hyx[n] * L : 0;
                    const R mz = zs ? a.psi_hyz[n] + s.cpsi_hyz[n] * L : 0;
                    if (xs) a.psi_hyx[n] = s.b_mx[i] * mx;
                    if (zs) a.psi_hyz[n] = s.b_mz[k] * mz;
                    const R gz = s.Chyez[n] * L + (xs ? s.a_mx[i] * mx : 0);
                    const R gx = s.Chyex[n] * L + (zs ? s.a_mz[k] * mz : 0);
                    a.ez[n + sx] += gz; a.ez[n] -= gz;
                    a.ex[n + sz] += gx; a.ex[n] -= gx;
                    a.hy[n] = s.Chyh[n] * L;
                }
                if (i < NX - 1 && j < NY - 1) {  // Hz
                    const R L = a.hz[n];
                    const R mx = xs ? a.psi_hzx[n] + s.cpsi_hzx[n] * L : 0;
                    const R my = ys ? a.psi_hzy[n] + s.cpsi_hzy[n] * L : 0;
                    if (xs) a.psi_hzx[n] = s.b_mx[i] * mx;
                    if (ys) a.psi_hzy[n] = s.b_my[j] * my;
                    const R gx = s.Chzex[n] * L + (ys ? s.a_my[j] * my : 0);
                    const R gy = s.Chzey[n] * L + (xs ? s.a_mx[i] * mx : 0);
                    a.ex[n + sy] += gx; a.ex[n] -= gx;
                    a.ey[n + sx] += gy; a.ey[n] -= gy;
                    a.hz[n] = s.Chzh[n] * L;
                }
            }
}

template <class R>
void reverse_e(const Sim<R>& s, Adj<R>& a) {
    const int NX = s.NX, NY = s.NY, NZ = s.NZ;
    const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const size_t n = s.id(i, j, k);
                const bool xs = (i > 0 && i < s.pxn) || (i > NX - s.pxp - 1 && i < NX - 1);
                const bool ys = (j > 0 && j < s.pyn) || (j > NY - s.pyp - 1 && j < NY - 1);
                const bool zs = (k > 0 && k < s.pzn) || (k > NZ - s.pzp - 1 && k < NZ - 1);
                if (i < NX - 1 && j > 0 && j < NY - 1 && k > 0 && k < NZ - 1) {  // Ex
                    const R L = a.ex[n];
                    const R my = ys ? a.psi_exy[n] + s.cpsi_exy[n] * L : 0;
                    const R mz = zs ? a.psi_exz[n] + s.cpsi_exz[n] * L : 0;
                    if (ys) a.psi_exy[n] = s.b_ey[j] * my;
                    if (zs) a.psi_exz[n] = s.b_ez[k] * mz;
                    const R gz = s.Cexhz[n] * L + (ys ? s.a_ey[j] * my : 0);
                    const R gy = s.Cexhy[n] * L + (zs ? s.a_ez[k] * mz : 0);
                    a.hz[n] += gz; a.hz[n - sy] -= gz;
                    a.hy[n] += gy; a.hy[n - sz] -= gy;
                    a.ex[n] = s.Cexe[n] * L;
                }
                if (i > 0 && i < NX - 1 && j < NY - 1 && k > 0 && k < NZ - 1) {  // Ey
                    const R L = a.ey[n];
                    const R mx = xs ? a.psi_eyx[n] + s.cpsi_eyx[n] * L : 0;
                    const R mz = zs ? a.psi_eyz[n] + s.cpsi_eyz[n] * L : 0;
                    if (xs) a.psi_eyx[n] = s.b_ex[i] * mx;
                    if (zs) a.psi_eyz[n] = s.b_ez[k] * mz;
                    const R gx = s.Ceyhx[n] * L + (zs ? s.a_ez[k] * mz : 0);
                    const R gz = s.Ceyhz[n] * L + (xs ? s.a_ex[i] * mx : 0);
                    a.hx[n] += gx; a.hx[n - sz] -= gx;
                    a.hz[n] += gz; a.hz[n - sx] -= gz;
                    a.ey[n] = s.Ceye[n] * L;
                }
                if (i > 0 && i < NX - 1 && j > 0 && j < NY - 1 && k < NZ - 1) {  // Ez
                    const R L = a.ez[n];
                    const R mx = xs ? a.psi_ezx[n] + s.cpsi_ezx[n] * L : 0;
                    const R my = ys ? a.psi_ezy[n] + s.cpsi_ezy[n] * L : 0;
                    if (xs) a.psi_ezx[n] = s.b_ex[i] * mx;
                    if (ys) a.psi_ezy[n] = s.b_ey[j] * my;
                    const R gy = s.Cezhy[n] * L + (xs ? s.a_ex[i] * mx : 0);
                    const R gx = s.Cezhx[n] * L + (ys ? s.a_ey[j] * my : 0);
                    a.hy[n] += gy; a.hy[n - sx] -= gy;
                    a.hx[n] += gx; a.hx[n - sy] -= gx;
                    a.ez[n] = s.Ceze[n] * L;
                }
            }
}

// dJ/deps_r of the design cells: for every E edge whose four surrounding cells touch the design
// region, lambda(edge) * dE'/d(eps_avg), shared as 1/4 by each surrounding cell. E^m, H^m are the
// fields before the step; lam the adjoint of E^{m+1}. Coefficients from the averaged eps/sigma.
template <class R>
void accumulate_grad(const Sim<R>& s, const Adj<R>& a, const std::vector<R>* Em[3], const std::vector<R>* Hm[3],
                     const int* d, double* grad) {
    const int NX = s.NX, NY = s.NY, NZ = s.NZ;
    const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
    const int gx = d[3] - d[0], gy = d[4] - d[1];
    auto add = [&](int ci, int cj, int ck, double v) {
        if (ci < d[0] || ci >= d[3] || cj < d[1] || cj >= d[4] || ck < d[2] || ck >= d[5]) return;
        grad[((size_t)(ck - d[2]) * gy + (cj - d[1])) * gx + (ci - d[0])] += 0.25 * v;
    };
    const R two = 2, four = 4;
    for (int k = std::max(d[2], 1); k <= std::min(d[5], NZ - 2); ++k)
        for (int j = std::max(d[1], 1); j <= std::min(d[4], NY - 2); ++j)
            for (int i = std::max(d[0], 1); i <= std::min(d[3], NX - 2); ++i) {
                const size_t n = s.id(i, j, k);
                {   // Ex(i,j,k): cells (i,j,k) (i,j-1,k) (i,j,k-1) (i,j-1,k-1)
                    const R den = two * s.eps_x[n] * s.eps0 + s.dt * s.sig_x[n];
                    const R dca = four * s.eps0 * s.dt * s.sig_x[n] / (den * den);
                    const R curl = s.Cexhz[n] * ((*Hm[2])[n] - (*Hm[2])[n - sy]) + s.Cexhy[n] * ((*Hm[1])[n] - (*Hm[1])[n - sz]);
                    const double v = (double)(a.ex[n] * (dca * (*Em[0])[n] - two * s.eps0 / den * curl));
                    add(i, j, k, v); add(i, j - 1, k, v); add(i, j, k - 1, v); add(i, j - 1, k - 1, v);
                }
                {   // Ey(i,j,k): cells (i,j,k) (i-1,j,k) (i,j,k-1) (i-1,j,k-1)
                    const R den = two * s.eps_y[n] * s.eps0 + s.dt * s.sig_y[n];
                    const R dca = four * s.eps0 * s.dt * s.sig_y[n] / (den * den);
                    const R curl = s.Ceyhx[n] * ((*Hm[0])[n] - (*Hm[0])[n - sz]) + s.Ceyhz[n] * ((*Hm[2])[n] - (*Hm[2])[n - sx]);
                    const double v = (double)(a.ey[n] * (dca * (*Em[1])[n] - two * s.eps0 / den * curl));
                    add(i, j, k, v); add(i - 1, j, k, v); add(i, j, k - 1, v); add(i - 1, j, k - 1, v);
                }
                {   // Ez(i,j,k): cells (i,j,k) (i-1,j,k) (i,j-1,k) (i-1,j-1,k)
                    const R den = two * s.eps_z[n] * s.eps0 + s.dt * s.sig_z[n];
                    const R dca = four * s.eps0 * s.dt * s.sig_z[n] / (den * den);
                    const R curl = s.Cezhy[n] * ((*Hm[1])[n] - (*Hm[1])[n - sx]) + s.Cezhx[n] * ((*Hm[0])[n] - (*Hm[0])[n - sy]);
                    const double v = (double)(a.ez[n] * (dca * (*Em[2])[n] - two * s.eps0 / den * curl));
                    add(i, j, k, v); add(i - 1, j, k, v); add(i, j - 1, k, v); add(i - 1, j - 1, k, v);
                }
            }
}

// FoM and (optionally) its adjoint gradient. Stores the whole field history (small grids only).
template <class R>
int fom_and_grad(const or_scenario* sc, int steps, const float* sig, int n_sig, int pi, int pj, int pk,
                 double* J_out, double* grad_out) {
    Sim<R> s;
    if (setup<R>(s, sc, sig, n_sig)) return -1;
    const size_t n_p = s.id(pi, pj, pk);
    std::vector<R> row(std::max<size_t>(s.probes.size(), 1));
    std::vector<std::vector<R>> hist;  // E^m, H^m for m = 0..steps-1 (6 arrays each) when needed
    std::vector<R> ezp(steps);
    for (int m = 0; m < steps; ++m) {
        if (grad_out)
            for (int c = 0; c < 6; ++c) hist.push_back(*field(s, c));
        calc_e<R>(s, m, row.data());
        ezp[m] = s.Ez[n_p];  // Ez after step m's E update (probe outside the CPML)
        calc_h<R>(s, row.data());
    }
    const double dt = (double)s.dt;
    double J = 0;
    for (int m = 0; m < steps; ++m) J += dt * (double)ezp[m] * (double)ezp[m];
    *J_out = J;
    if (!grad_out) return 0;
    const int* d = sc->design_box;
    std::fill(grad_out, grad_out + (size_t)(d[3] - d[0]) * (d[4] - d[1]) * (d[5] - d[2]), 0.0);
    Adj<R> a(s.N);
    for (int m = steps - 1; m >= 0; --m) {
        a.ez[n_p] += (R)(2.0 * dt) * ezp[m];  // dJ/dEz(p) of the sample taken in step m
        reverse_h<R>(s, a);
        const std::vector<R>* Em[3] = {&hist[6 * m + 0], &hist[6 * m + 1], &hist[6 * m + 2]};
        const std::vector<R>* Hm[3] = {&hist[6 * m + 3], &hist[6 * m + 4], &hist[6 * m + 5]};
        accumulate_grad<R>(s, a, Em, Hm, d, grad_out);
        reverse_e<R>(s, a);
    }
    return 0;
}

// fom_and_grad for long runs: the forward keeps, per step, only the fields of the design region's
// nodes and of the node layer below it (all accumulate_grad reads) instead of the whole history,
// and the reverse sweep writes them back into full-volume scratch arrays before each gradient
// step. Same arithmetic, same result; memory (steps x 6 x box nodes) instead of (steps x 6 x N).
template <class R>
int fom_and_grad_box(const or_scenario* sc, int steps, const float* sig, int n_sig, int pi, int pj, int pk,
                     double* J_out, double* grad_out) {
    Sim<R> s;
    if (setup<R>(s, sc, sig, n_sig)) return -1;
    const size_t n_p = s.id(pi, pj, pk);
    const int* d = sc->design_box;
    const int i0 = std::max(d[0] - 1, 0), i1 = std::min(d[3], s.NX - 1);
    const int j0 = std::max(d[1] - 1, 0), j1 = std::min(d[4], s.NY - 1);
    const int k0 = std::max(d[2] - 1, 0), k1 = std::min(d[5], s.NZ - 1);
    const size_t bx = (size_t)(i1 - i0 + 1), by = (size_t)(j1 - j0 + 1), bz = (size_t)(k1 - k0 + 1);
    const size_t nb = bx * by * bz;
    auto box_copy = [&](R* box, std::vector<R>& full, bool to_box) {
        size_t q = 0;
        for (int k = k0; k <= k1; ++k)
            for (int j = j0; j <= j1; ++j)
                for (int i = i0; i <= i1; ++i, ++q) {
                    const size_t n = s.id(i, j, k);
                    if (to_box) box[q] = full[n];
                    else full[n] = box[q];
                }
    };
    std::vector<R> row(std::max<size_t>(s.probes.size(), 1));
    std::vector<R> hist(grad_out ? (size_t)steps * 6 * nb : 0);
    std::vector<R> ezp(steps);
    for (int m = 0; m < steps; ++m) {
        if (grad_out)
            for (int c = 0; c < 6; ++c) box_copy(&hist[((size_t)m * 6 + c) * nb], *field(s, c), true);
        calc_e<R>(s, m, row.data());
        ezp[m] = s.Ez[n_p];
        calc_h<R>(s, row.data());
    }
    const double dt = (double)s.dt;
    double J = 0;
    for (int m = 0; m < steps; ++m) J += dt * (double)ezp[m] * (double)ezp[m];
    *J_out = J;
    if (!grad_out) return 0;
    std::fill(grad_out, grad_out + (size_t)(d[3] - d[0]) * (d[4] - d[1]) * (d[5] - d[2]), 0.0);
    std::vector<R> scratch[6];
    for (auto& v : scratch) v.assign(s.N, (R)0);
    const std::vector<R>* Em[3] = {&scratch[0], &scratch[1], &scratch[2]};
    const std::vector<R>* Hm[3] = {&scratch[3], &scratch[4], &scratch[5]};
    Adj<R> a(s.N);
    for (int m = steps - 1; m >= 0; --m) {
        a.ez[n_p] += (R)(2.0 * dt) * ezp[m];
        reverse_h<R>(s, a);
        for (int c = 0; c < 6; ++c) box_copy(&hist[((size_t)m * 6 + c) * nb], scratch[c], false);
        accumulate_grad<R>(s, a, Em, Hm, d, grad_out);
        reverse_e<R>(s, a);
    }
    return 0;
}

}  // namespace

extern "C" {

// FP64 figure of merit J = sum_m dt Ez(pi,pj,pk)^2 and, when grad is non-NULL, dJ/deps_r over the
// scenario's design region (from the discrete adjoint).
int or_fom_grad_f64(const or_scenario* sc, int steps, const float* sig, int n_sig, int pi, int pj, int pk,
                    double* J, double* grad) {
    return fom_and_grad<double>(sc, steps, sig, n_sig, pi, pj, pk, J, grad);
}
int or_fom_grad_f32(const or_scenario* sc, int steps, const float* sig, int n_sig, int pi, int pj, int pk,
                    double* J, double* grad) {
    return fom_and_grad<float>(sc, steps, sig, n_sig, pi, pj, pk, J, grad);
}
// or_fom_grad_f64 keeping only the design region's field history (long runs, large grids).
int or_fom_grad_box_f64(const or_scenario* sc, int steps, const float* sig, int n_sig, int pi, int pj, int pk,
                        double* J, double* grad) {
    return fom_and_grad_box<double>(sc, steps, sig, n_sig, pi, pj, pk, J, grad);
}

// Seconds the time loop of the last or_run_f32 / or_run_f64 took (setup excluded).
double or_last_step_seconds(void) { return g_last_step_seconds; }

// Full run: probes_out (steps, nprobe), fields_out (6, nz, ny, nx). signal_per_node (nsrc, n_sig).
int or_run_f32(const or_scenario* sc, int steps, const float* sig, int n_sig, const float* init_fields,
               float* probes_out, float* fields_out, int nthreads) {
    return run<float>(sc, steps, sig, n_sig, init_fields, probes_out, fields_out, nthreads, -1);
}
int or_run_f64(const or_scenario* sc, int steps, const float* sig, int n_sig, const float* init_fields,
               double* probes_out, double* fields_out, int nthreads) {
    return run<double>(sc, steps, sig, n_sig, init_fields, probes_out, fields_out, nthreads, -1);
}
// One calc_e (fields_out[0..2] after it) then one calc_h (fields_out[3..5]) from init_fields.
// init_psi / psi_out: 12 (nz,ny,nx) arrays in the order eyx, ezx, exy, ezy, exz, eyz, hyx, hzx,
// hxy, hzy, hxz, hyz (either may be NULL).
int or_onestep_f32(const or_scenario* sc, int m, const float* sig, int n_sig, const float* init_fields,
                   float* fields_out, const float* init_psi, float* psi_out) {
    return run<float>(sc, 0, sig, n_sig, init_fields, nullptr, fields_out, 1, m, init_psi, psi_out);
}

// Port voltage and current from sampled series (steps rows of `stride` floats, the port's columns
// from col0): the voltage box's Ez samples (k outer, then j, then i; the range along the voltage
// direction `vaxis` half-open, the others closed), then four groups of H samples s1..s4 of the
// current loop for current direction `axis` (0 x, 1 y, 2 z; the groups of fdtd_gb300's
// port_groups, in summation order). Restates voltMgpu cases 1-3 (fdtdrav.h:2214-2290): a float
// sum in that order times csuf = -dx / ((je-js+1)(ke-ks+1)), -dy / ((ke-ks+1)(ie-is+1)) or
// -dz / ((ie-is+1)(je-js+1));
// currMgpu cases 1-3 (fdtdrav.h:2318-2480): four float sums and a1*s1 + a2*s2 - a1*s3 - a2*s4
// (a1, a2 = dy, dz / dz, dx / dy, dx), contracted as the reference's compiled expressions are
// (x loop: a1*s1 fused with a2*s2 as the addend; y, z loops: a2*s2 fused with a1*s1 as the
// addend; then two FMAs; found by comparing the candidate contractions against the reference's
// outputs); and, with time_average, correcI
// (fdtdrav.h:2490-2508) in the order its in-place threads produced their results.
int or_port_vi(const float* series, int steps, int stride, int col0, const int* vbox, const int* cbox, int axis,
               int vaxis, float dx, float dy, float dz, int time_average, float* V, float* I) {
    // voltMgpu (fdtdrav.h:2214-2290): the Ez samples of the box, half-open along the voltage axis
    const int nv = (vbox[3] - vbox[0] + (vaxis == 0 ? 0 : 1)) * (vbox[4] - vbox[1] + (vaxis == 1 ? 0 : 1)) *
                   (vbox[5] - vbox[2] + (vaxis == 2 ? 0 : 1));
    const int ni = cbox[3] - cbox[0] + 1, nj = cbox[4] - cbox[1] + 1, nk = cbox[5] - cbox[2] + 1;
    int n[4];
    float a1, a2;
    if (axis == 0) { n[0] = nj; n[1] = nk; n[2] = nj; n[3] = nk; a1 = dy; a2 = dz; }
    else if (axis == 1) { n[0] = nk; n[1] = ni; n[2] = nk; n[3] = ni; a1 = dz; a2 = dx; }
    else { n[0] = nj; n[1] = ni; n[2] = nj; n[3] = ni; a1 = dy; a2 = dx; }
    if (nv <= 0 || ni <= 0 || nj <= 0 || nk <= 0 || col0 + nv + n[0] + n[1] + n[2] + n[3] > stride) {
        g_err = "port columns outside the series";
        return -1;
    }
    const float is = (float)vbox[0], js = (float)vbox[1], ks = (float)vbox[2];
    const float ie = (float)vbox[3], je = (float)vbox[4], ke = (float)vbox[5];
    const float csuf = vaxis == 0   ? (-dx) / ((je - js + 1) * (ke - ks + 1))
                       : vaxis == 1 ? (-dy) / ((ke - ks + 1) * (ie - is + 1))
                                    : (-dz) / ((ie - is + 1) * (je - js + 1));
    for (int t = 0; t < steps; ++t) {
        const float* r = series + (size_t)t * stride + col0;
        float v = 0.f;
        for (int q = 0; q < nv; ++q) v = v + r[q];
        V[t] = v * csuf;
        const float* hs = r + nv;
        float sum[4];
        for (int g = 0; g < 4; ++g) {
            float acc = 0.f;
            for (int q = 0; q < n[g]; ++q) acc = acc + hs[q];
            sum[g] = acc;
            hs += n[g];
        }
        const float lead = axis == 0 ? std::fmaf(a1, sum[0], a2 * sum[1]) : std::fmaf(a2, sum[1], a1 * sum[0]);
        I[t] = std::fmaf(-a2, sum[3], std::fmaf(-a1, sum[2], lead));
    }
    if (time_average && steps > 1) {
        // each step from its unaveraged successor; the last step from its averaged predecessor
        // (the order in which the reference's in-place kernel produced its results)
        std::vector<float> raw(I, I + steps);
        for (int t = 0; t + 1 < steps; ++t) I[t] = (raw[t] + raw[t + 1]) / 2;
        I[steps - 1] = (raw[steps - 1] + I[steps - 2]) / 2;
    }
    return 0;
}

// Per-edge coefficient arrays after the full setup, by reference name (volume (nz,ny,nx) or 1-D).
int or_coef_f32(const or_scenario* sc, const char* name, float* out) {
    Sim<float> s;
    static const float zero = 0.f;
    if (setup<float>(s, sc, &zero, 0)) return -1;
    std::string n(name);
#define GETV(v) if (n == #v) { std::memcpy(out, s.v.data(), s.v.size() * sizeof(float)); return 0; }
    VEC_LIST(GETV)
    GETV(eps_x) GETV(eps_y) GETV(eps_z) GETV(sig_x) GETV(sig_y) GETV(sig_z)
    GETV(mu_x) GETV(mu_y) GETV(mu_z) GETV(sm_x) GETV(sm_y) GETV(sm_z)
    GETV(b_ex) GETV(a_ex) GETV(b_mx) GETV(a_mx) GETV(b_ey) GETV(a_ey) GETV(b_my) GETV(a_my)
    GETV(b_ez) GETV(a_ez) GETV(b_mz) GETV(a_mz)
#undef GETV
    g_err = "unknown array " + n;
    return -1;
}

}  // extern "C"
