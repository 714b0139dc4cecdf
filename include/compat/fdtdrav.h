/* Drop-in declaration of the reference's whole-run entry point, for its driver.
 *
 * The reference's driver (source.cu) includes "fdtdrav.h" and calls marchingLoop (source.cu:297);
 * fdtdrav.h defines that function (fdtdrav.h:3425-4387) with every kernel behind it. Compiled with
 * this directory first on the include path (-I include/compat) and linked against
 * libfdtd_gb300.so, the unchanged driver runs the same scenario on this library instead: the
 * function below has marchingLoop's exact parameter list and C++ linkage, runs the whole domain
 * on the current device through the C ABI (fdtd_marching_loop, fdtd_api.h), and writes V(t) and
 * the time-averaged I(t) to results1003.dat and results1004.dat in the working directory, one
 * "%e \n" line per step, as the reference's saveTDomain does (fdtdrav.h:2704-2719, 4364-4367).
 * Unlike the reference it never exits the process: an error is printed to stderr (with
 * fdtd_last_error's text) and no result file is written. */
#ifndef FDTD_COMPAT_FDTDRAV_H
#define FDTD_COMPAT_FDTDRAV_H

#ifndef __cplusplus
#error "marchingLoop has C++ linkage, as in the reference"
#endif

void marchingLoop(const int NUMDEV, float eps_0, float pi, float mu_0, float c, float dx, float dy, float dz, float dt,
                  int X, int Y, int Z,
                  int n_t_steps,
                  int pml_x_n, int pml_y_n, int pml_z_n, int pml_x_p, int pml_y_p, int pml_z_p,
                  int air_buff_x_n, int air_buff_y_n, int air_buff_z_n, int air_buff_x_p, int air_buff_y_p, int air_buff_z_p,
                  int source_tp, float source_freq, float source_amp,
                  float source_min_x, float source_min_y, float source_min_z,
                  float source_max_x, float source_max_y, float source_max_z,
                  int source_direction, float rs, float nc, float tau, float t_0,
                  float* brick_min_x, float* brick_min_y, float* brick_min_z,
                  float* brick_max_x, float* brick_max_y, float* brick_max_z,
                  float* brick_sigma_e_x, float* brick_sigma_e_y, float* brick_sigma_e_z,
                  float* brick_eps_r_x, float* brick_eps_r_y, float* brick_eps_r_z,
                  float* brick_sigma_m_x, float* brick_sigma_m_y, float* brick_sigma_m_z,
                  float* brick_mu_r_x, float* brick_mu_r_y, float* brick_mu_r_z,
                  int brick_opt, int brick_num,
                  float* pec_min_x, float* pec_min_y, float* pec_min_z,
                  float* pec_max_x, float* pec_max_y, float* pec_max_z,
                  float* pec_sigma_e_x, float* pec_sigma_e_y, float* pec_sigma_e_z,
                  int pec_opt, int pec_num,
                  float resistor_min_x, float resistor_min_y, float resistor_min_z,
                  float resistor_max_x, float resistor_max_y, float resistor_max_z,
                  float resistor_resist, int resistor_direction, int resistor_opt,
                  float sampled_voltage_min_x, float sampled_voltage_min_y, float sampled_voltage_min_z,
                  float sampled_voltage_max_x, float sampled_voltage_max_y, float sampled_voltage_max_z,
                  int voltage_direction,
                  float sampled_current_min_x, float sampled_current_min_y, float sampled_current_min_z,
                  float sampled_current_max_x, float sampled_current_max_y, float sampled_current_max_z,
                  int current_direction);

#endif /* FDTD_COMPAT_FDTDRAV_H */
