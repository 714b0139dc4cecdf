// A driver in the shape of the reference's source.cu: includes "fdtdrav.h" (resolved to
// include/compat/fdtdrav.h) and calls marchingLoop with every parameter by position, linked
// against libfdtd_gb300.so. The parameter values come from a text file written by
// tests/test_gpu_marching.py ("name value" lines; arrays "name n v0 .. vn-1"), so the test can
// compare the result files with the reference pipeline's V(t) and I(t).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "fdtdrav.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: marching_driver params.txt\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::map<std::string, double> s;
    std::map<std::string, std::vector<float>> a;
    std::string name, kind;
    while (in >> name >> kind) {
        if (kind == "a") {
            size_t n = 0;
            in >> n;
            std::vector<float>& v = a[name];
            v.resize(n > 0 ? n : 1, 0.f);
            for (size_t q = 0; q < n; ++q) in >> v[q];
        } else {
            in >> s[name];
        }
    }
    auto I = [&](const char* k) { return (int)s.at(k); };
    auto F = [&](const char* k) { return (float)s.at(k); };
    auto A = [&](const char* k) { return a.at(k).data(); };
    marchingLoop(I("NUMDEV"), F("eps_0"), F("pi"), F("mu_0"), F("c"), F("dx"), F("dy"), F("dz"), F("dt"),
                 I("X"), I("Y"), I("Z"),
                 I("n_t_steps"),
                 I("pml_x_n"), I("pml_y_n"), I("pml_z_n"), I("pml_x_p"), I("pml_y_p"), I("pml_z_p"),
                 I("air_buff_x_n"), I("air_buff_y_n"), I("air_buff_z_n"), I("air_buff_x_p"), I("air_buff_y_p"),
                 I("air_buff_z_p"),
                 I("source_tp"), F("source_freq"), F("source_amp"),
                 F("source_min_x"), F("source_min_y"), F("source_min_z"),
                 F("source_max_x"), F("source_max_y"), F("source_max_z"),
                 I("source_direction"), F("rs"), F("nc"), F("tau"), F("t_0"),
                 A("brick_min_x"), A("brick_min_y"), A("brick_min_z"),
                 A("brick_max_x"), A("brick_max_y"), A("brick_max_z"),
                 A("brick_sigma_e_x"), A("brick_sigma_e_y"), A("brick_sigma_e_z"),
                 A("brick_eps_r_x"), A("brick_eps_r_y"), A("brick_eps_r_z"),
                 A("brick_sigma_m_x"), A("brick_sigma_m_y"), A("brick_sigma_m_z"),
                 A("brick_mu_r_x"), A("brick_mu_r_y"), A("brick_mu_r_z"),
                 I("brick_opt"), I("brick_num"),
                 A("pec_min_x"), A("pec_min_y"), A("pec_min_z"),
                 A("pec_max_x"), A("pec_max_y"), A("pec_max_z"),
                 A("pec_sigma_e_x"), A("pec_sigma_e_y"), A("pec_sigma_e_z"),
                 I("pec_opt"), I("pec_num"),
                 F("resistor_min_x"), F("resistor_min_y"), F("resistor_min_z"),
                 F("resistor_max_x"), F("resistor_max_y"), F("resistor_max_z"),
                 F("resistor_resist"), I("resistor_direction"), I("resistor_opt"),
                 F("sampled_voltage_min_x"), F("sampled_voltage_min_y"), F("sampled_voltage_min_z"),
                 F("sampled_voltage_max_x"), F("sampled_voltage_max_y"), F("sampled_voltage_max_z"),
                 I("voltage_direction"),
                 F("sampled_current_min_x"), F("sampled_current_min_y"), F("sampled_current_min_z"),
                 F("sampled_current_max_x"), F("sampled_current_max_y"), F("sampled_current_max_z"),
                 I("current_direction"));
    std::printf("End of Program\n");
    return 0;
}
