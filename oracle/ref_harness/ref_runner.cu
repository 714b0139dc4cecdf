// Host-side runner for the reference kernels (test infrastructure only; never part of the product).
//
// Loads the cubin built from the reference's fdtdrav.h (see ref_kernels.cu and oracle/build_ref.sh),
// allocates the reference's 84 per-cell arrays plus its 1-D CPML arrays and ghost planes for a
// single slab (NUMDEV = 1, gpu_offset = 0), and drives the reference's setup kernels in the order
// of marchingLoop (fdtdrav.h:4047-4310) followed by calc_e then calc_h per step (solver,
// fdtdrav.h:3222-3333). Launch shapes follow fdtdrav.h:3714-3720: block (16,16,4), NX and NY padded
// to multiples of 16 (fdtdrav.h:3493-3494).
//
// Differences from marchingLoop, all on the host side:
//  * the scenario comes in as index-space boxes instead of metres (the metre->index mapping,
//    calc_index fdtdrav.h:198-206, is restated in fdtd_gb300/scenario.py);
//  * sizes are computed in size_t (the reference computes byte counts in float, fdtdrav.h:3700);
//  * several lumped sources may be defined (defineSourceZ once per box); calc_e injects only the
//    one whose box is passed to it, so multi-source runs are done once per source and summed;
//  * the per-node source signal is supplied by the caller instead of setGauss/setSine;
//  * the reference's own sample boxes are placed outside the grid and a gather kernel of ours
//    records probe values after every step.
// Every error is returned as a status code with a message; nothing exits the process.

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include <vector>
#include <map>
#include <algorithm>

namespace {

std::string g_err;
cudaLibrary_t g_lib = nullptr;

struct Kern { const char* name; cudaKernel_t k; };
enum { K_SETZERO, K_SETBRICK, K_SETSIGMA, K_SETCOEF, K_SETABCPML, K_SRCZ, K_RES, K_CALCE, K_CALCH,
       K_VOLT, K_CURR, K_CORREC, K_PLATEX, K_PLATEY, K_PLATEZ, K_GAUSS, K_SINE, K_SEC, K_SRCX, K_ZIN, K_GATHER,
       K_COUNT };
Kern g_k[K_COUNT] = {
    {"_Z7setZero", nullptr}, {"_Z8setBrick", nullptr}, {"_Z18setSigmaEpsSigmaMu", nullptr},
    {"_Z15setCoefficients", nullptr}, {"_Z9setABCPML", nullptr}, {"_Z13defineSourceZ", nullptr},
    {"_Z14defineResistor", nullptr}, {"_Z6calc_e", nullptr}, {"_Z6calc_h", nullptr},
    {"_Z8voltMgpu", nullptr}, {"_Z8currMgpu", nullptr}, {"_Z7correcI", nullptr},
    {"_Z12definePlateX", nullptr}, {"_Z12definePlateY", nullptr}, {"_Z12definePlateZ", nullptr},
    {"_Z8setGauss", nullptr}, {"_Z7setSine", nullptr}, {"_Z9defineSec", nullptr}, {"_Z13defineSourceX", nullptr},
    {"_Z8c_zinS11P6float2S0_iS0_S0_S0_S0_S_f", nullptr}, {"harness_gather", nullptr}};

// Itanium-ABI names of the reference kernels: the parameter lists of fdtdrav.h reduce to runs of
// int (i), float (f) and float* (Pf, then the substitution S_).
std::string mangled(const char* prefix, const char* spec) {
    // spec: sequence of <count><code>, code in {i, f, p}; the first p emits Pf, the rest S_.
    std::string out(prefix);
    bool seen_p = false;
    const char* s = spec;
    while (*s) {
        int n = 0;
        while (*s >= '0' && *s <= '9') n = n * 10 + (*s++ - '0');
        char c = *s++;
        for (int r = 0; r < n; ++r) {
            if (c == 'i') out += "i";
            else if (c == 'f') out += "f";
            else { out += seen_p ? "S_" : "Pf"; seen_p = true; }
        }
    }
    return out;
}

struct Dims { int NX, NXX, NY, NYY, NZ, NZ_N; int pml[6]; float dx, dy, dz, dt, eps0, pi, mu0; };
Dims g_d;
bool g_ready = false;

// All reference arrays by name. Volume arrays hold NX*NY*NZ floats, 1-D CPML arrays hold
// max(NX, NY, NZ) floats, ghost planes NX*NY floats.
std::map<std::string, float*> g_arr;
std::vector<std::string> g_order;
size_t g_vol = 0, g_line = 0, g_plane = 0;
float* g_gather_fields = nullptr;  // device array of 6 pointers (float**)
float* g_probe_dev = nullptr;
int* g_probe_comp_dev = nullptr;
long long* g_probe_idx_dev = nullptr;
float* g_signal_dev = nullptr;
size_t g_signal_cap = 0;
int g_probe_cap = 0;

std::vector<std::vector<int>> g_src_box;

// The reference's own voltage / current sample boxes (calc_e / calc_h arguments). Outside the grid
// unless rh_set_port placed them; g_port_steps bounds the time index the sample arrays hold.
int g_vbox[6] = {-10, -10, -10, -10, -10, -10}, g_vn[3] = {1, 1, 1};
int g_cbox[6] = {-10, -10, -10, -10, -10, -10}, g_cn[3] = {1, 1, 1};
int g_port_steps = 0;

const char* kVolumeNames[] = {
    "Ex", "Jx", "Cexe", "Cexhz", "Cexhy", "Cexj", "eps_r_x", "sigma_e_x",
    "Ey", "Jy", "Ceye", "Ceyhx", "Ceyhz", "Ceyj", "eps_r_y", "sigma_e_y",
    "Ez", "Jz", "Ceze", "Cezhy", "Cezhx", "Cezj", "eps_r_z", "sigma_e_z",
    "Hx", "Mx", "Chxh", "Chxey", "Chxez", "Chxm", "mu_r_x", "sigma_m_x",
    "Hy", "My", "Chyh", "Chyez", "Chyex", "Chym", "mu_r_y", "sigma_m_y",
    "Hz", "Mz", "Chzh", "Chzex", "Chzey", "Chzm", "mu_r_z", "sigma_m_z",
    "mat_eps_x", "mat_eps_y", "mat_eps_z", "mat_sigma_e_x", "mat_sigma_e_y", "mat_sigma_e_z",
    "mat_mu_x", "mat_mu_y", "mat_mu_z", "mat_sigma_m_x", "mat_sigma_m_y", "mat_sigma_m_z",
    "Psi_eyx", "Psi_ezx", "Psi_hyx", "Psi_hzx", "cpsi_eyx", "cpsi_ezx", "cpsi_hyx", "cpsi_hzx",
    "Psi_exy", "Psi_ezy", "Psi_hxy", "Psi_hzy", "cpsi_exy", "cpsi_ezy", "cpsi_hxy", "cpsi_hzy",
    "Psi_exz", "Psi_eyz", "Psi_hxz", "Psi_hyz", "cpsi_exz", "cpsi_eyz", "cpsi_hxz", "cpsi_hyz"};
const char* kLineNames[] = {"cpml_b_ex", "cpml_a_ex", "cpml_b_mx", "cpml_a_mx",
                            "cpml_b_ey", "cpml_a_ey", "cpml_b_my", "cpml_a_my",
                            "cpml_b_ez", "cpml_a_ez", "cpml_b_mz", "cpml_a_mz"};
const char* kPlaneNames[] = {"gEx", "gEy", "gHx", "gHy"};
const char* kSampleNames[] = {"sampE", "sampHx", "sampHy", "sampHz"};

float* A(const char* n) { return g_arr.at(n); }

bool ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        g_err = std::string(what) + ": " + cudaGetErrorString(e);
        return false;
    }
    return true;
}

dim3 grid3d() { return dim3(g_d.NX / 16, g_d.NY / 16, (g_d.NZ_N + 3) / 4); }
dim3 block3d() { return dim3(16, 16, 4); }

bool launch(int kid, dim3 g, dim3 b, std::vector<void*>& args) {
    cudaError_t e = cudaLaunchKernel((const void*)g_k[kid].k, g, b, args.data(), 0, 0);
    return ck(e, g_k[kid].name);
}

void free_all() {
    for (auto& kv : g_arr) cudaFree(kv.second);
    g_arr.clear();
    g_order.clear();
    if (g_gather_fields) cudaFree(g_gather_fields);
    if (g_probe_dev) cudaFree(g_probe_dev);
    if (g_probe_comp_dev) cudaFree(g_probe_comp_dev);
    if (g_probe_idx_dev) cudaFree(g_probe_idx_dev);
    if (g_signal_dev) cudaFree(g_signal_dev);
    g_gather_fields = nullptr; g_probe_dev = nullptr; g_probe_comp_dev = nullptr;
    g_probe_idx_dev = nullptr; g_signal_dev = nullptr; g_signal_cap = 0; g_probe_cap = 0;
    g_ready = false;
    for (int q = 0; q < 6; ++q) g_vbox[q] = g_cbox[q] = -10;
    for (int q = 0; q < 3; ++q) g_vn[q] = g_cn[q] = 1;
    g_port_steps = 0;
}

}  // namespace

extern "C" {

typedef struct {
    int nxx, nyy, nz;
    int pml[6];  // x_n, x_p, y_n, y_p, z_n, z_p
    float dx, dy, dz, dt, eps0, pi, mu0;
    // box is,js,ks,ie,je,ke; material (nbricks, 3, 4): per axis x, y, z eps_r, sigma_e, mu_r, sigma_m
    int nbricks; const int* brick_box; const float* brick_mat;
    int nsources; const int* src_box; const float* src_r;       // box is,js,ks,ie,je,ke
    int nres; const int* res_box; const float* res_r;
    int nplates; const int* plate; const float* plate_sig;  // (n, 7): axis, box; (n, 2): sigma_e pair
    int nsrcx; const int* srcx_box; const float* srcx_r;     // defineSourceX boxes and resistances
} rh_scenario;

const char* rh_error(void) { return g_err.c_str(); }

int rh_load(const char* cubin_path) {
    if (g_lib) return 0;
    if (!ck(cudaLibraryLoadFromFile(&g_lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0),
            "cudaLibraryLoadFromFile")) return -1;
    const char* specs[K_COUNT] = {
        "96p3i",                       // setZero
        "5i12p6i12f",                  // setBrick
        "5i24p",                       // setSigmaEpsSigmaMu
        "7i36p7f",                     // setCoefficients
        "7i36p13f",                    // setABCPML
        "13i6p6f",                     // defineSourceZ
        "14i5p6f",                     // defineResistor
        "14i57p16i1p",                 // calc_e
        "13i56p10i3p",                 // calc_h
        "11i2p3f2i",                   // voltMgpu
        "11i4p3f2i",                   // currMgpu
        "1p1i",                        // correcI
        "5i2p2f6i",                    // definePlateX
        "5i2p2f6i",                    // definePlateY
        "5i2p2f6i",                    // definePlateZ
        "2p1f1i3f1i",                  // setGauss
        "2p1i4f1i",                    // setSine
        "14i3f2p3f",                   // defineSec
        "13i6p6f",                     // defineSourceX
        nullptr, nullptr};             // c_zinS11 (float2 parameters, full name above), gather
    for (int k = 0; k < K_COUNT; ++k) {
        std::string nm = (k < K_COUNT && specs[k]) ? mangled(g_k[k].name, specs[k]) : std::string(g_k[k].name);
        if (!ck(cudaLibraryGetKernel(&g_k[k].k, g_lib, nm.c_str()), nm.c_str())) return -1;
    }
    return 0;
}

int rh_setup(const rh_scenario* s) {
    if (!g_lib) { g_err = "rh_load not called"; return -1; }
    free_all();
    Dims d;
    d.NXX = s->nxx; d.NYY = s->nyy; d.NZ = s->nz;
    d.NX = (d.NXX % 16 == 0) ? d.NXX : (d.NXX / 16 + 1) * 16;
    d.NY = (d.NYY % 16 == 0) ? d.NYY : (d.NYY / 16 + 1) * 16;
    d.NZ_N = d.NZ;
    for (int q = 0; q < 6; ++q) d.pml[q] = s->pml[q];
    d.dx = s->dx; d.dy = s->dy; d.dz = s->dz; d.dt = s->dt; d.eps0 = s->eps0; d.pi = s->pi; d.mu0 = s->mu0;
    g_d = d;
    g_vol = (size_t)d.NX * d.NY * d.NZ;
    g_line = (size_t)std::max(d.NX, std::max(d.NY, d.NZ));
    g_plane = (size_t)d.NX * d.NY;
    for (const char* n : kVolumeNames) {
        float* p = nullptr;
        if (!ck(cudaMalloc(&p, g_vol * sizeof(float)), "cudaMalloc volume")) { free_all(); return -1; }
        g_arr[n] = p; g_order.push_back(n);
    }
    for (const char* n : kLineNames) {
        float* p = nullptr;
        if (!ck(cudaMalloc(&p, g_line * sizeof(float)), "cudaMalloc line")) { free_all(); return -1; }
        g_arr[n] = p; g_order.push_back(n);
    }
    for (const char* n : kPlaneNames) {
        float* p = nullptr;
        if (!ck(cudaMalloc(&p, g_plane * sizeof(float)), "cudaMalloc plane")) { free_all(); return -1; }
        cudaMemset(p, 0, g_plane * sizeof(float));
        g_arr[n] = p; g_order.push_back(n);
    }
    for (const char* n : kSampleNames) {  // never written: the sample boxes lie outside the grid
        float* p = nullptr;
        if (!ck(cudaMalloc(&p, 64 * sizeof(float)), "cudaMalloc sample")) { free_all(); return -1; }
        g_arr[n] = p; g_order.push_back(n);
    }
    {
        float* ptrs[6] = {A("Ex"), A("Ey"), A("Ez"), A("Hx"), A("Hy"), A("Hz")};
        if (!ck(cudaMalloc(&g_gather_fields, sizeof(ptrs)), "cudaMalloc gather")) { free_all(); return -1; }
        cudaMemcpy(g_gather_fields, ptrs, sizeof(ptrs), cudaMemcpyHostToDevice);
    }
    int NX = d.NX, NXX = d.NXX, NY = d.NY, NYY = d.NYY, NZ = d.NZ, NZ_N = d.NZ_N, off = 0;

    // setZero (fdtdrav.h:919), argument order of fdtdrav.h:4047-4067
    {
        std::vector<void*> a;
        static float* P[96];
        const char* order[] = {
            "Ex", "Jx", "Cexe", "Cexhz", "Cexhy", "Cexj", "eps_r_x", "sigma_e_x",
            "Ey", "Jy", "Ceye", "Ceyhx", "Ceyhz", "Ceyj", "eps_r_y", "sigma_e_y",
            "Ez", "Jz", "Ceze", "Cezhy", "Cezhx", "Cezj", "eps_r_z", "sigma_e_z",
            "Hx", "Mx", "Chxh", "Chxey", "Chxez", "Chxm", "mu_r_x", "sigma_m_x",
            "Hy", "My", "Chyh", "Chyez", "Chyex", "Chym", "mu_r_y", "sigma_m_y",
            "Hz", "Mz", "Chzh", "Chzex", "Chzey", "Chzm", "mu_r_z", "sigma_m_z",
            "mat_eps_x", "mat_eps_y", "mat_eps_z", "mat_sigma_e_x", "mat_sigma_e_y", "mat_sigma_e_z",
            "mat_mu_x", "mat_mu_y", "mat_mu_z", "mat_sigma_m_x", "mat_sigma_m_y", "mat_sigma_m_z",
            "cpml_b_ex", "cpml_a_ex", "cpml_b_mx", "cpml_a_mx",
            "cpml_b_ey", "cpml_a_ey", "cpml_b_my", "cpml_a_my",
            "cpml_b_ez", "cpml_a_ez", "cpml_b_mz", "cpml_a_mz",
            "Psi_eyx", "Psi_ezx", "Psi_hyx", "Psi_hzx", "cpsi_eyx", "cpsi_ezx", "cpsi_hyx", "cpsi_hzx",
            "Psi_exy", "Psi_ezy", "Psi_hxy", "Psi_hzy", "cpsi_exy", "cpsi_ezy", "cpsi_hxy", "cpsi_hzy",
            "Psi_exz", "Psi_eyz", "Psi_hxz", "Psi_hyz", "cpsi_exz", "cpsi_eyz", "cpsi_hxz", "cpsi_hyz"};
        for (int q = 0; q < 96; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
        a.push_back(&NX); a.push_back(&NY); a.push_back(&NZ_N);
        if (!launch(K_SETZERO, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // setBrick per box (fdtdrav.h:1524, called at 4104-4128)
    for (int b = 0; b < s->nbricks; ++b) {
        const int* bx = s->brick_box + 6 * b;
        const float* bm = s->brick_mat + 12 * b;
        int is = bx[0], js = bx[1], ks = bx[2], ie = bx[3], je = bx[4], ke = bx[5];
        // setBrick's value order: sigma_e, eps_r, sigma_m, mu_r, each x, y, z
        static float v[12];
        for (int a = 0; a < 3; ++a) {
            v[a] = bm[4 * a + 1]; v[3 + a] = bm[4 * a]; v[6 + a] = bm[4 * a + 3]; v[9 + a] = bm[4 * a + 2];
        }
        static float* P[12];
        const char* order[] = {"mat_eps_x", "mat_eps_y", "mat_eps_z", "mat_sigma_e_x", "mat_sigma_e_y", "mat_sigma_e_z",
                               "mat_mu_x", "mat_mu_y", "mat_mu_z", "mat_sigma_m_x", "mat_sigma_m_y", "mat_sigma_m_z"};
        std::vector<void*> a = {&NX, &NY, &NZ, &NZ_N, &off};
        for (int q = 0; q < 12; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
        a.push_back(&is); a.push_back(&js); a.push_back(&ks); a.push_back(&ie); a.push_back(&je); a.push_back(&ke);
        for (int q = 0; q < 12; ++q) a.push_back(&v[q]);
        if (!launch(K_SETBRICK, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // setSigmaEpsSigmaMu (fdtdrav.h:1097, called at 4133-4150)
    {
        static float* P[24];
        const char* order[] = {"mat_eps_x", "mat_eps_y", "mat_eps_z", "mat_sigma_e_x", "mat_sigma_e_y", "mat_sigma_e_z",
                               "mat_mu_x", "mat_mu_y", "mat_mu_z", "mat_sigma_m_x", "mat_sigma_m_y", "mat_sigma_m_z",
                               "eps_r_x", "sigma_e_x", "eps_r_y", "sigma_e_y", "eps_r_z", "sigma_e_z",
                               "mu_r_x", "sigma_m_x", "mu_r_y", "sigma_m_y", "mu_r_z", "sigma_m_z"};
        std::vector<void*> a = {&NX, &NY, &NZ, &NZ_N, &off};
        for (int q = 0; q < 24; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
        if (!launch(K_SETSIGMA, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // definePlateX / Y / Z per plate, in order (fdtdrav.h:1574-1679, called at 4162-4182)
    for (int q = 0; q < s->nplates; ++q) {
        const int* pl = s->plate + 7 * q;
        int is = pl[1], js = pl[2], ks = pl[3], ie = pl[4], je = pl[5], ke = pl[6];
        float sa = s->plate_sig[2 * q], sb = s->plate_sig[2 * q + 1];
        static float* P[2];
        const int kid = pl[0] == 0 ? K_PLATEX : pl[0] == 1 ? K_PLATEY : K_PLATEZ;
        if (pl[0] == 0) { P[0] = A("sigma_e_y"); P[1] = A("sigma_e_z"); }
        else if (pl[0] == 1) { P[0] = A("sigma_e_x"); P[1] = A("sigma_e_z"); }
        else { P[0] = A("sigma_e_x"); P[1] = A("sigma_e_y"); }
        std::vector<void*> a = {&NX, &NY, &NZ, &NZ_N, &off, &P[0], &P[1], &sa, &sb,
                                &is, &js, &ks, &ie, &je, &ke};
        if (!launch(kid, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // setCoefficients (fdtdrav.h:1223, called at 4213-4230)
    {
        static float* P[36];
        const char* order[] = {
            "Cexe", "Cexhz", "Cexhy", "Cexj", "eps_r_x", "sigma_e_x",
            "Ceye", "Ceyhx", "Ceyhz", "Ceyj", "eps_r_y", "sigma_e_y",
            "Ceze", "Cezhy", "Cezhx", "Cezj", "eps_r_z", "sigma_e_z",
            "Chxh", "Chxey", "Chxez", "Chxm", "mu_r_x", "sigma_m_x",
            "Chyh", "Chyez", "Chyex", "Chym", "mu_r_y", "sigma_m_y",
            "Chzh", "Chzex", "Chzey", "Chzm", "mu_r_z", "sigma_m_z"};
        std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off};
        for (int q = 0; q < 36; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
        a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&g_d.dt);
        a.push_back(&g_d.eps0); a.push_back(&g_d.pi); a.push_back(&g_d.mu0);
        if (!launch(K_SETCOEF, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // setABCPML (fdtdrav.h:1747, called at 4237-4258); the pml sizes are float parameters there
    {
        static float* P[36];
        static float pf[6];
        const char* order[] = {
            "cpml_b_ex", "cpml_a_ex", "cpml_b_mx", "cpml_a_mx", "cpml_b_ey", "cpml_a_ey", "cpml_b_my", "cpml_a_my",
            "cpml_b_ez", "cpml_a_ez", "cpml_b_mz", "cpml_a_mz",
            "cpsi_eyx", "cpsi_ezx", "cpsi_hyx", "cpsi_hzx", "cpsi_exy", "cpsi_ezy", "cpsi_hxy", "cpsi_hzy",
            "cpsi_exz", "cpsi_eyz", "cpsi_hxz", "cpsi_hyz",
            "Cexhz", "Cexhy", "Ceyhx", "Ceyhz", "Cezhy", "Cezhx", "Chxey", "Chxez", "Chyez", "Chyex", "Chzex", "Chzey"};
        std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off};
        for (int q = 0; q < 36; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
        // call order: pml_x_n, pml_y_n, pml_z_n, pml_x_p, pml_y_p, pml_z_p (fdtdrav.h:4255)
        pf[0] = (float)d.pml[0]; pf[1] = (float)d.pml[2]; pf[2] = (float)d.pml[4];
        pf[3] = (float)d.pml[1]; pf[4] = (float)d.pml[3]; pf[5] = (float)d.pml[5];
        for (int q = 0; q < 6; ++q) a.push_back(&pf[q]);
        a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&g_d.dt);
        a.push_back(&g_d.eps0); a.push_back(&g_d.pi); a.push_back(&g_d.mu0);
        if (!launch(K_SETABCPML, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // defineSourceZ per source (fdtdrav.h:1368, called at 4275-4277)
    g_src_box.clear();
    for (int q = 0; q < s->nsources; ++q) {
        const int* bx = s->src_box + 6 * q;
        g_src_box.push_back(std::vector<int>(bx, bx + 6));
        int is = bx[0], js = bx[1], ks = bx[2], ie = bx[3], je = bx[4], ke = bx[5];
        float rs = s->src_r[q];
        static float* P[6];
        const char* order[] = {"Ceze", "Cezhy", "Cezhx", "Cezj", "eps_r_z", "sigma_e_z"};
        std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off, &is, &js, &ks, &ie, &je, &ke};
        for (int r = 0; r < 6; ++r) { P[r] = A(order[r]); a.push_back(&P[r]); }
        a.push_back(&rs); a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&g_d.dt);
        a.push_back(&g_d.eps0);
        if (!launch(K_SRCZ, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // defineSourceX per x-directed element (fdtdrav.h:1311, called at 4278 for source_direction 1)
    for (int q = 0; q < s->nsrcx; ++q) {
        const int* bx = s->srcx_box + 6 * q;
        int is = bx[0], js = bx[1], ks = bx[2], ie = bx[3], je = bx[4], ke = bx[5];
        float rs = s->srcx_r[q];
        static float* P[6];
        const char* order[] = {"Cexe", "Cexhz", "Cexhy", "Cexj", "eps_r_x", "sigma_e_x"};
        std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off, &is, &js, &ks, &ie, &je, &ke};
        for (int r = 0; r < 6; ++r) { P[r] = A(order[r]); a.push_back(&P[r]); }
        a.push_back(&rs); a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&g_d.dt);
        a.push_back(&g_d.eps0);
        if (!launch(K_SRCX, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    // defineResistor per resistor (fdtdrav.h:1429, called at 4295-4309)
    for (int q = 0; q < s->nres; ++q) {
        const int* bx = s->res_box + 6 * q;
        int is = bx[0], js = bx[1], ks = bx[2], ie = bx[3], je = bx[4], ke = bx[5], dir = 3;
        float rs = s->res_r[q];
        static float* P[5];
        const char* order[] = {"Ceze", "Cezhy", "Cezhx", "eps_r_z", "sigma_e_z"};
        std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off, &is, &js, &ks, &ie, &je, &ke, &dir};
        for (int r = 0; r < 5; ++r) { P[r] = A(order[r]); a.push_back(&P[r]); }
        a.push_back(&rs); a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&g_d.dt);
        a.push_back(&g_d.eps0);
        if (!launch(K_RES, grid3d(), block3d(), a)) { free_all(); return -1; }
    }
    if (!ck(cudaDeviceSynchronize(), "setup sync")) { free_all(); return -1; }
    g_ready = true;
    return 0;
}

// Copy a reference array to the host. Volume arrays are returned as the (nz, nyy, nxx) region
// (x fastest), 1-D arrays as their first `len` entries.
int rh_get(const char* name, float* out, long long len) {
    auto it = g_arr.find(name);
    if (it == g_arr.end()) { g_err = std::string("unknown array ") + name; return -1; }
    bool vol = false;
    for (const char* n : kVolumeNames) vol |= (strcmp(n, name) == 0);
    if (!vol) return ck(cudaMemcpy(out, it->second, (size_t)len * sizeof(float), cudaMemcpyDeviceToHost), "rh_get") ? 0 : -1;
    for (int k = 0; k < g_d.NZ; ++k)  // rows of one z-plane are contiguous, planes are NX*NY apart
        if (!ck(cudaMemcpy2D(out + (size_t)k * g_d.NXX * g_d.NYY, (size_t)g_d.NXX * sizeof(float),
                             it->second + (size_t)k * g_plane, (size_t)g_d.NX * sizeof(float),
                             (size_t)g_d.NXX * sizeof(float), (size_t)g_d.NYY, cudaMemcpyDeviceToHost), "rh_get 2D"))
            return -1;
    return 0;
}

// Overwrite a volume array's (nz, nyy, nxx) region from the host (used to seed random states).
int rh_set(const char* name, const float* in) {
    auto it = g_arr.find(name);
    if (it == g_arr.end()) { g_err = std::string("unknown array ") + name; return -1; }
    for (int k = 0; k < g_d.NZ; ++k)
        if (!ck(cudaMemcpy2D(it->second + (size_t)k * g_plane, (size_t)g_d.NX * sizeof(float),
                             in + (size_t)k * g_d.NXX * g_d.NYY, (size_t)g_d.NXX * sizeof(float),
                             (size_t)g_d.NXX * sizeof(float), (size_t)g_d.NYY, cudaMemcpyHostToDevice), "rh_set 2D"))
            return -1;
    return 0;
}

static bool ensure_signal(const float* sig, long long n) {
    if ((size_t)n > g_signal_cap) {
        if (g_signal_dev) cudaFree(g_signal_dev);
        g_signal_dev = nullptr;
        if (!ck(cudaMalloc(&g_signal_dev, (size_t)n * sizeof(float)), "cudaMalloc signal")) return false;
        g_signal_cap = (size_t)n;
    }
    return ck(cudaMemcpy(g_signal_dev, sig, (size_t)n * sizeof(float), cudaMemcpyHostToDevice), "signal H2D");
}

static bool do_calc_e(int m, int src_slot) {
    int NX = g_d.NX, NXX = g_d.NXX, NY = g_d.NY, NYY = g_d.NYY, NZ = g_d.NZ, NZ_N = g_d.NZ_N, off = 0, voff = 0;
    int* pml = g_d.pml;  // x_n, x_p, y_n, y_p, z_n, z_p (calc_e parameter order)
    static int sbox[6];
    if (src_slot >= 0) for (int q = 0; q < 6; ++q) sbox[q] = g_src_box[src_slot][q];
    else { sbox[0] = sbox[1] = sbox[2] = -10; sbox[3] = sbox[4] = sbox[5] = -10; }
    static int vbox[6], vn[3];
    for (int q = 0; q < 6; ++q) vbox[q] = g_vbox[q];
    for (int q = 0; q < 3; ++q) vn[q] = g_vn[q];
    static float* P[57];
    const char* order[] = {
        "Ex", "Jx", "Cexe", "Cexhz", "Cexhy", "Cexj", "Ey", "Jy", "Ceye", "Ceyhx", "Ceyhz", "Ceyj",
        "Ez", "Jz", "Ceze", "Cezhy", "Cezhx", "Cezj", "Hx", "Mx", "Hy", "My", "Hz", "Mz", "gHx", "gHy",
        "cpml_b_ex", "cpml_a_ex", "cpml_b_ey", "cpml_a_ey", "cpml_b_ez", "cpml_a_ez",
        "Psi_eyx", "Psi_ezx", "Psi_hyx", "Psi_hzx", "cpsi_eyx", "cpsi_ezx", "cpsi_hyx", "cpsi_hzx",
        "Psi_exy", "Psi_ezy", "Psi_hxy", "Psi_hzy", "cpsi_exy", "cpsi_ezy", "cpsi_hxy", "cpsi_hzy",
        "Psi_exz", "Psi_eyz", "Psi_hxz", "Psi_hyz", "cpsi_exz", "cpsi_eyz", "cpsi_hxz", "cpsi_hyz"};
    std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off, &voff};
    for (int q = 0; q < 6; ++q) a.push_back(&pml[q]);
    for (int q = 0; q < 56; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
    P[56] = g_signal_dev ? g_signal_dev : A("sampE");
    a.push_back(&P[56]);
    for (int q = 0; q < 6; ++q) a.push_back(&sbox[q]);
    for (int q = 0; q < 6; ++q) a.push_back(&vbox[q]);
    for (int q = 0; q < 3; ++q) a.push_back(&vn[q]);
    static int mm; mm = m; a.push_back(&mm);
    static float* PE; PE = A("sampE"); a.push_back(&PE);
    return launch(K_CALCE, grid3d(), block3d(), a);
}

static bool do_calc_h(int m) {
    int NX = g_d.NX, NXX = g_d.NXX, NY = g_d.NY, NYY = g_d.NYY, NZ = g_d.NZ, NZ_N = g_d.NZ_N, off = 0;
    int* pml = g_d.pml;
    static int cbox[6], cn[3];
    for (int q = 0; q < 6; ++q) cbox[q] = g_cbox[q];
    for (int q = 0; q < 3; ++q) cn[q] = g_cn[q];
    static float* P[56];
    const char* order[] = {
        "Ex", "Jx", "Ey", "Jy", "Ez", "Jz", "gEx", "gEy",
        "Hx", "Mx", "Chxh", "Chxey", "Chxez", "Chxm", "Hy", "My", "Chyh", "Chyez", "Chyex", "Chym",
        "Hz", "Mz", "Chzh", "Chzex", "Chzey", "Chzm",
        "cpml_b_mx", "cpml_a_mx", "cpml_b_my", "cpml_a_my", "cpml_b_mz", "cpml_a_mz",
        "Psi_eyx", "Psi_ezx", "Psi_hyx", "Psi_hzx", "cpsi_eyx", "cpsi_ezx", "cpsi_hyx", "cpsi_hzx",
        "Psi_exy", "Psi_ezy", "Psi_hxy", "Psi_hzy", "cpsi_exy", "cpsi_ezy", "cpsi_hxy", "cpsi_hzy",
        "Psi_exz", "Psi_eyz", "Psi_hxz", "Psi_hyz", "cpsi_exz", "cpsi_eyz", "cpsi_hxz", "cpsi_hyz"};
    std::vector<void*> a = {&NX, &NXX, &NY, &NYY, &NZ, &NZ_N, &off};
    for (int q = 0; q < 6; ++q) a.push_back(&pml[q]);
    for (int q = 0; q < 56; ++q) { P[q] = A(order[q]); a.push_back(&P[q]); }
    for (int q = 0; q < 6; ++q) a.push_back(&cbox[q]);
    for (int q = 0; q < 3; ++q) a.push_back(&cn[q]);
    static int mm; mm = m; a.push_back(&mm);
    static float* PH[3]; PH[0] = A("sampHx"); PH[1] = A("sampHy"); PH[2] = A("sampHz");
    a.push_back(&PH[0]); a.push_back(&PH[1]); a.push_back(&PH[2]);
    return launch(K_CALCH, grid3d(), block3d(), a);
}

// One reference E half-step (calc_e) at time index m with source slot src_slot (-1: none).
int rh_calc_e(int m, int src_slot, const float* signal, long long nsig) {
    if (!g_ready) { g_err = "not set up"; return -1; }
    if (g_port_steps > 0) { g_err = "single half-steps are not used with a port"; return -1; }
    if (signal && !ensure_signal(signal, nsig)) return -1;
    if (!do_calc_e(m, src_slot)) return -1;
    return ck(cudaDeviceSynchronize(), "calc_e sync") ? 0 : -1;
}

int rh_calc_h(int m) {
    if (!g_ready) { g_err = "not set up"; return -1; }
    if (g_port_steps > 0) { g_err = "single half-steps are not used with a port"; return -1; }
    if (!do_calc_h(m)) return -1;
    return ck(cudaDeviceSynchronize(), "calc_h sync") ? 0 : -1;
}

// Run n_steps reference steps m0 .. m0+n_steps-1 (calc_e then calc_h each step). If nprobes > 0,
// probe values (component 0..5 = Ex,Ey,Ez,Hx,Hy,Hz at node i,j,k) are gathered after each step
// into probe_out[step][probe]. elapsed_ms receives the device time of the whole loop (CUDA events).
int rh_run(int m0, int n_steps, int src_slot, const float* signal, long long nsig,
           int nprobes, const int* pcomp, const int* pi, const int* pj, const int* pk,
           float* probe_out, float* elapsed_ms) {
    if (!g_ready) { g_err = "not set up"; return -1; }
    if (g_port_steps > 0 && (m0 < 0 || m0 + n_steps > g_port_steps)) { g_err = "steps beyond the port sample arrays"; return -1; }
    if (signal && !ensure_signal(signal, nsig)) return -1;
    if (nprobes > 0) {
        if (nprobes > g_probe_cap) {
            if (g_probe_comp_dev) cudaFree(g_probe_comp_dev);
            if (g_probe_idx_dev) cudaFree(g_probe_idx_dev);
            g_probe_comp_dev = nullptr; g_probe_idx_dev = nullptr;
            if (!ck(cudaMalloc(&g_probe_comp_dev, nprobes * sizeof(int)), "probe comp") ||
                !ck(cudaMalloc(&g_probe_idx_dev, nprobes * sizeof(long long)), "probe idx")) return -1;
            g_probe_cap = nprobes;
        }
        std::vector<long long> idx(nprobes);
        for (int p = 0; p < nprobes; ++p)
            idx[p] = (long long)pi[p] + (long long)pj[p] * g_d.NX + (long long)pk[p] * g_d.NX * g_d.NY;
        cudaMemcpy(g_probe_comp_dev, pcomp, nprobes * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(g_probe_idx_dev, idx.data(), nprobes * sizeof(long long), cudaMemcpyHostToDevice);
        if (g_probe_dev) cudaFree(g_probe_dev);
        g_probe_dev = nullptr;
        if (!ck(cudaMalloc(&g_probe_dev, (size_t)nprobes * n_steps * sizeof(float)), "probe buf")) return -1;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    for (int m = m0; m < m0 + n_steps; ++m) {
        if (!do_calc_e(m, src_slot)) return -1;
        if (!do_calc_h(m)) return -1;
        if (nprobes > 0) {
            float* outp = g_probe_dev + (size_t)(m - m0) * nprobes;
            std::vector<void*> a = {&g_gather_fields, &g_probe_comp_dev, &g_probe_idx_dev, &outp, &nprobes};
            if (!launch(K_GATHER, dim3((nprobes + 127) / 128), dim3(128), a)) return -1;
        }
    }
    cudaEventRecord(e1, 0);
    if (!ck(cudaEventSynchronize(e1), "run sync")) return -1;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (elapsed_ms) *elapsed_ms = ms;
    if (nprobes > 0 && probe_out)
        if (!ck(cudaMemcpy(probe_out, g_probe_dev, (size_t)nprobes * n_steps * sizeof(float), cudaMemcpyDeviceToHost),
                "probe D2H")) return -1;
    return 0;
}

long long rh_padded_dims(int* nx, int* ny) { *nx = g_d.NX; *ny = g_d.NY; return (long long)g_vol; }

void rh_free(void) { free_all(); }

// The reference's source waveform kernels as marchingLoop launches them (fdtdrav.h:4068-4086,
// 1-D blocks of 512): type 1 setGauss, type 3 setSine. Returns d_signal and d_signal_per_node.
int rh_waveform(int type, float amp, int v_mag_factor, float freq, float dt, float t_0, float tau, float pi, int n,
                float* signal, float* per_node) {
    if (!g_lib) { g_err = "rh_load not called"; return -1; }
    if (type != 1 && type != 3) { g_err = "waveform type 1 or 3"; return -1; }
    float *ds = nullptr, *dn = nullptr;
    if (!ck(cudaMalloc(&ds, n * sizeof(float)), "cudaMalloc signal") ||
        !ck(cudaMalloc(&dn, n * sizeof(float)), "cudaMalloc per node")) { cudaFree(ds); return -1; }
    int block = 512, grid = n / block + ((n % block) == 0 ? 0 : 1);
    std::vector<void*> a;
    if (type == 1) a = {&ds, &dn, &amp, &v_mag_factor, &dt, &t_0, &tau, &n};
    else a = {&ds, &dn, &v_mag_factor, &amp, &freq, &dt, &pi, &n};
    bool ok = launch(type == 1 ? K_GAUSS : K_SINE, dim3(grid), dim3(block), a) && ck(cudaDeviceSynchronize(), "waveform sync") &&
              ck(cudaMemcpy(signal, ds, n * sizeof(float), cudaMemcpyDeviceToHost), "signal D2H") &&
              ck(cudaMemcpy(per_node, dn, n * sizeof(float), cudaMemcpyDeviceToHost), "per node D2H");
    cudaFree(ds); cudaFree(dn);
    return ok ? 0 : -1;
}

static bool realloc_sample(const char* name, size_t n) {
    float*& p = g_arr[name];
    if (p) cudaFree(p);
    p = nullptr;
    if (!ck(cudaMalloc(&p, n * sizeof(float)), "cudaMalloc port sample")) return false;
    return ck(cudaMemset(p, 0, n * sizeof(float)), "memset port sample");
}

// Place the reference's voltage and current sample boxes (z-directed port, fdtdrav.h:3628-3652
// sizes) for runs of at most n_steps steps starting at m = 0. Boxes are checked to lie inside the
// grid with the current box's low x / y neighbours, so every sampleField write stays in bounds.
int rh_set_port(const int* vbox, const int* cbox, int n_steps) {
    if (!g_ready) { g_err = "not set up"; return -1; }
    const int* v = vbox; const int* c = cbox;
    if (n_steps < 2 || v[0] < 0 || v[3] >= g_d.NXX || v[0] > v[3] || v[1] < 0 || v[4] >= g_d.NYY || v[1] > v[4] ||
        v[2] < 0 || v[5] >= g_d.NZ || v[2] >= v[5] || c[0] < 1 || c[3] >= g_d.NXX || c[0] > c[3] || c[1] < 1 ||
        c[4] >= g_d.NYY || c[1] > c[4] || c[2] < 1 || c[5] >= g_d.NZ || c[2] > c[5]) {
        g_err = "port boxes outside the grid"; return -1;
    }
    int vnx = v[3] - v[0] + 1, vny = v[4] - v[1] + 1, cnx = c[3] - c[0] + 2, cny = c[4] - c[1] + 2;
    if (!realloc_sample("sampE", (size_t)vnx * vny * g_d.NZ_N * n_steps)) return -1;
    for (const char* n : {"sampHx", "sampHy", "sampHz"})
        if (!realloc_sample(n, (size_t)cnx * cny * g_d.NZ_N * n_steps)) return -1;
    for (int q = 0; q < 6; ++q) { g_vbox[q] = v[q]; g_cbox[q] = c[q]; }
    g_vn[0] = vnx; g_vn[1] = vny; g_vn[2] = g_d.NZ_N;
    g_cn[0] = cnx; g_cn[1] = cny; g_cn[2] = g_d.NZ_N;
    g_port_steps = n_steps;
    return 0;
}

// The reference's port reductions on its own samples, launched as calcVoltCurrent does
// (fdtdrav.h:3129-3186, NUMDEV = 1, 1-D blocks of 512): voltMgpu (voltage_direction 1, 2 or 3)
// and currMgpu (current_direction 1, 2 or 3), then correcI in place. Returns V(t), I(t) before
// correcI and I(t) after it.
int rh_port_reduce_dir(int n_steps, int voltage_direction, int current_direction, float* volt, float* curr_raw,
                       float* curr_avg);
int rh_port_reduce(int n_steps, int current_direction, float* volt, float* curr_raw, float* curr_avg) {
    return rh_port_reduce_dir(n_steps, 3, current_direction, volt, curr_raw, curr_avg);
}
int rh_port_reduce_dir(int n_steps, int voltage_direction, int current_direction, float* volt, float* curr_raw,
                       float* curr_avg) {
    if (g_port_steps <= 0 || n_steps != g_port_steps) { g_err = "rh_set_port first, same n_steps"; return -1; }
    float *dv = nullptr, *di = nullptr;
    if (!ck(cudaMalloc(&dv, n_steps * sizeof(float)), "cudaMalloc V") ||
        !ck(cudaMalloc(&di, n_steps * sizeof(float)), "cudaMalloc I")) { cudaFree(dv); return -1; }
    int block = 512, grid = n_steps / block + ((n_steps % block) == 0 ? 0 : 1);
    int off = 0, dir = voltage_direction, cdir = current_direction, n = n_steps;
    if (cdir < 1 || cdir > 3 || dir < 1 || dir > 3) {
        g_err = "directions must be 1, 2 or 3"; cudaFree(dv); cudaFree(di); return -1;
    }
    static int vb[6], cb[6], vn[4], cn[4];
    for (int q = 0; q < 6; ++q) { vb[q] = g_vbox[q]; cb[q] = g_cbox[q]; }
    vn[0] = g_vn[0]; vn[1] = g_vn[1]; vn[2] = g_d.NZ; vn[3] = g_d.NZ_N;
    cn[0] = g_cn[0]; cn[1] = g_cn[1]; cn[2] = g_d.NZ; cn[3] = g_d.NZ_N;
    static float* P[5];
    bool ok = true;
    {
        P[0] = dv; P[1] = A("sampE");
        std::vector<void*> a = {&vn[0], &vn[1], &vn[2], &vn[3], &off};
        for (int q = 0; q < 6; ++q) a.push_back(&vb[q]);
        a.push_back(&P[0]); a.push_back(&P[1]);
        a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&n); a.push_back(&dir);
        ok = ok && launch(K_VOLT, dim3(grid), dim3(block), a);
    }
    {
        P[0] = di; P[2] = A("sampHx"); P[3] = A("sampHy"); P[4] = A("sampHz");
        std::vector<void*> a = {&cn[0], &cn[1], &cn[2], &cn[3], &off};
        for (int q = 0; q < 6; ++q) a.push_back(&cb[q]);
        a.push_back(&P[0]); a.push_back(&P[2]); a.push_back(&P[3]); a.push_back(&P[4]);
        a.push_back(&g_d.dx); a.push_back(&g_d.dy); a.push_back(&g_d.dz); a.push_back(&n); a.push_back(&cdir);
        ok = ok && launch(K_CURR, dim3(grid), dim3(block), a);
    }
    ok = ok && ck(cudaDeviceSynchronize(), "port reduce sync") &&
         ck(cudaMemcpy(volt, dv, n_steps * sizeof(float), cudaMemcpyDeviceToHost), "V D2H") &&
         ck(cudaMemcpy(curr_raw, di, n_steps * sizeof(float), cudaMemcpyDeviceToHost), "I D2H");
    if (ok) {
        std::vector<void*> a = {&P[0], &n};
        ok = launch(K_CORREC, dim3(grid), dim3(block), a) && ck(cudaDeviceSynchronize(), "correcI sync") &&
             ck(cudaMemcpy(curr_avg, di, n_steps * sizeof(float), cudaMemcpyDeviceToHost), "I avg D2H");
    }
    cudaFree(dv); cudaFree(di);
    return ok ? 0 : -1;
}

// The reference's defineSec (fdtdrav.h:1681-1744) on the set-up handle's averaged sigma_e_x /
// sigma_e_y arrays, launched as marchingLoop's sector loop would (fdtdrav.h:4175, grid3d, block3d,
// NUMDEV = 1); tri = {px0, py0, px1, py1, px2, py2}. Read the arrays back with rh_get.
int rh_sector(const int* tri, int pz0, float raio, int max_x, int max_y, float sx, float sy) {
    if (!g_ready) { g_err = "not set up"; return -1; }
    int NX = g_d.NX, NY = g_d.NY, NZ = g_d.NZ, NZ_N = g_d.NZ_N, off = 0, mx = max_x, my = max_y;
    int t[6] = {tri[0], tri[1], tri[2], tri[3], tri[4], tri[5]};
    int z = pz0;
    float r = raio, a = sx, b = sy, dx = g_d.dx, dy = g_d.dy, dz = g_d.dz;
    static float* P[2];
    P[0] = A("sigma_e_x");
    P[1] = A("sigma_e_y");
    std::vector<void*> args = {&NX, &NY, &NZ, &NZ_N, &off, &mx, &my, &t[0], &t[1], &t[2], &t[3], &t[4], &t[5], &z,
                               &r, &a, &b, &P[0], &P[1], &dx, &dy, &dz};
    return launch(K_SEC, grid3d(), block3d(), args) && ck(cudaDeviceSynchronize(), "defineSec sync") ? 0 : -1;
}

// The reference's c_zinS11 (fdtdrav.h:2510-2548) on given spectra of n_t_steps/2 + 1 bins
// (interleaved complex): returns s11 and zin, launched as calc_otm2 does (blocks of 1024).
int rh_zin(int n_t_steps, const float* V, const float* I, float z0_re, float z0_im, float* s11, float* zin) {
    if (!g_lib) { g_err = "rh_load not called"; return -1; }
    size_t nf = (size_t)n_t_steps / 2 + 1, bytes = nf * 2 * sizeof(float);
    float* d[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool ok = true;
    for (int q = 0; q < 6 && ok; ++q) ok = ck(cudaMalloc(&d[q], bytes), "cudaMalloc zin");
    ok = ok && ck(cudaMemcpy(d[0], V, bytes, cudaMemcpyHostToDevice), "V H2D") &&
         ck(cudaMemcpy(d[1], I, bytes, cudaMemcpyHostToDevice), "I H2D");
    if (ok) {
        int threads = 1024, grid = (int)((nf + threads - 1) / threads), n = n_t_steps;
        struct { float x, y; } z0 = {z0_re, z0_im};
        float dt = g_d.dt;
        std::vector<void*> a = {&d[0], &d[1], &n, &d[2], &d[3], &d[4], &d[5], &z0, &dt};
        ok = launch(K_ZIN, dim3(grid), dim3(threads), a) && ck(cudaDeviceSynchronize(), "zin sync") &&
             ck(cudaMemcpy(s11, d[4], bytes, cudaMemcpyDeviceToHost), "s11 D2H") &&
             ck(cudaMemcpy(zin, d[5], bytes, cudaMemcpyDeviceToHost), "zin D2H");
    }
    for (int q = 0; q < 6; ++q) cudaFree(d[q]);
    return ok ? 0 : -1;
}

}  // extern "C"
