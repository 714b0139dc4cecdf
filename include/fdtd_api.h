/* fdtd_api.h - C ABI of the GB300-native 3D FDTD solver (libfdtd_gb300.so).
 *
 * A single-domain, single-GPU replacement for the Yee time step of ravelec/FDTD and for the host
 * setup that feeds it. The reference has no plugin layer: its "API" is the host functions and
 * kernels of fdtdrav.h driven by marchingLoop (fdtdrav.h:3425-4387). Each entry point below names
 * the reference code it replaces.
 *
 * Conventions
 *  - Nodes are indexed (i, j, k), 0 <= i < nx, x fastest, exactly as the reference's
 *    idx = i + j*NX + k*NX*NY (fdtdrav.h:278); nx, ny, nz are the reference's NXX, NYY, NZ.
 *  - Host arrays are dense (nz, ny, nx) float32 / uint8, x fastest; the library pads rows itself.
 *  - All state is FP32. Every call returns FDTD_OK (0) or an error code and never exits the
 *    process; fdtd_last_error() returns the message of the calling thread's last failure.
 *  - One handle may be used by one host thread at a time; handles share no state.
 */
#ifndef FDTD_API_H
#define FDTD_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_OK 0
#define FDTD_ERR_INVALID 1   /* bad argument or configuration (checked on the host)          */
#define FDTD_ERR_CUDA 2      /* a CUDA runtime call failed                                   */
#define FDTD_ERR_OOM 3       /* device allocation failed                                     */
#define FDTD_ERR_STATE 4     /* call not allowed in the handle's current state               */
#define FDTD_ERR_RANGE 5     /* requested data outside what the handle holds                 */
#define FDTD_ERR_DEVICE 6    /* a kernel reported an error through its device status word     */

/* Field components. */
enum { FDTD_EX = 0, FDTD_EY = 1, FDTD_EZ = 2, FDTD_HX = 3, FDTD_HY = 4, FDTD_HZ = 5 };

/* Update-kernel schedules (fdtd_set_schedule). */
enum {
    FDTD_SCHEDULE_AUTO = 0,   /* two passes; on grids of >= 8 Mi cells the first fdtd_step call
                                 of >= 8 steps times 4 steps of each schedule and keeps the faster
                                 (that call synchronises the handle's stream) */
    FDTD_SCHEDULE_TWO_PASS = 1, /* E pass then H pass per step, in place (the reference's order) */
    FDTD_SCHEDULE_FUSED = 2,  /* one z-marching sweep per step over ping-pong field buffers   */
    FDTD_SCHEDULE_FUSED_CPML = 3 /* FUSED with the z-march also over the z and y CPML slabs and
                                    the boundary planes beside the interior tiles (slabs of at most
                                    15 cells, no design region); same bits, slower on the measured
                                    grids, so AUTO does not choose it */
};

typedef struct fdtd_handle fdtd_handle;

/* Grid and constants. Replaces the scalar parameters of marchingLoop (fdtdrav.h:3425-3430) after
 * its sizing (fdtdrav.h:3485-3498): nx/ny/nz are node counts including air buffer and CPML. */
typedef struct {
    int32_t nx, ny, nz;
    float dx, dy, dz, dt;
    float eps0, mu0, pi;     /* the reference passes these as floats (source.cu:30-33)      */
    int32_t pml[6];          /* CPML cells per face: x_n, x_p, y_n, y_p, z_n, z_p           */
} fdtd_grid;

/* One material: relative permittivity, electric conductivity (S/m), relative permeability,
 * magnetic conductivity. Replaces the per-brick scalars of setBrick (fdtdrav.h:1524-1571).
 * The background (material 0 by default) is eps_r = mu_r = 1, sigma = 1.2e-38 (setZero). */
typedef struct {
    float eps_r, sigma_e, mu_r, sigma_m;
} fdtd_material;

/* One material with separate values per axis (index 0 x, 1 y, 2 z): setBrick's brick_eps_r_x/y/z,
 * brick_sigma_e_x/y/z, brick_mu_r_x/y/z and brick_sigma_m_x/y/z (fdtdrav.h:1524-1531). A field
 * component averages the values of its own axis: Ex the x values of its four cells, Hx the x
 * values of its two cells, and so on (setSigmaEpsSigmaMu, fdtdrav.h:1097-1220). */
typedef struct {
    float eps_r[3], sigma_e[3], mu_r[3], sigma_m[3];
} fdtd_material_axes;

const char* fdtd_last_error(void);
const char* fdtd_version(void);

/* Allocate a simulation on the current CUDA device: fields set to 1.2e-38 (setZero,
 * fdtdrav.h:919-1094), material 0 everywhere. Replaces the allocation and initialisation part of
 * marchingLoop (fdtdrav.h:3874-4086). Validates the grid (CPML faces may not overlap). */
int fdtd_create(const fdtd_grid* grid, fdtd_handle** out);
/* Free everything the handle owns (the reference frees nothing, fdtdrav.h:4384). */
int fdtd_destroy(fdtd_handle* h);

/* Run all device work of this handle on a caller stream (a cudaStream_t); NULL = legacy stream. */
int fdtd_set_stream(fdtd_handle* h, void* cuda_stream);
int fdtd_set_schedule(fdtd_handle* h, int32_t schedule);
/* The schedule the next step runs: TWO_PASS or FUSED (AUTO resolved; -1 for a NULL handle). */
int32_t fdtd_active_schedule(const fdtd_handle* h);
/* Under AUTO, run the schedule trial now without advancing the handle: fields, CPML memory, probe
 * ring and step count are restored afterwards. Nothing to do for other schedules or a trial already
 * taken. Synchronises the handle's stream. */
int fdtd_tune_schedule(fdtd_handle* h);

/* Material table (at most 256 entries). Replaces the per-brick material scalars that setBrick
 * paints into 12 per-cell arrays (fdtdrav.h:1524-1571). */
int fdtd_set_materials(fdtd_handle* h, const fdtd_material* table, int32_t n);
/* The same with per-axis (anisotropic) materials, replacing the per-axis scalars of setBrick
 * (fdtdrav.h:1524-1571). */
int fdtd_set_materials_axes(fdtd_handle* h, const fdtd_material_axes* table, int32_t n);
/* Per-cell material index, host array of nz*ny*nx bytes (pinned memory copies fastest). Replaces
 * the painted per-cell material arrays; edge averaging (setSigmaEpsSigmaMu, fdtdrav.h:1097-1220)
 * is done on the fly. The indices are checked on the device after the copy: an index outside the
 * material table gives FDTD_ERR_INVALID and leaves every cell at material 0. */
int fdtd_set_material_index(fdtd_handle* h, const uint8_t* cells);
/* Paint cells [is,ie) x [js,je) x [ks,ke) with a material, last call wins (setBrick,
 * fdtdrav.h:1524-1571, called in order at fdtdrav.h:4104-4128). box = {is,js,ks,ie,je,ke}. */
int fdtd_add_brick(fdtd_handle* h, const int32_t box[6], int32_t material);

/* Lumped voltage source with internal resistance on the edges i in [is,ie], j in [js,je],
 * k in [ks,ke) (axis 2 = z, the only orientation the reference implements correctly).
 * voltage[m] is the source voltage at step m; each edge is driven with voltage[m]/(ke-ks)
 * (fdtdrav.h:1494, 3613). Replaces defineSourceZ (fdtdrav.h:1368-1426), setGauss/setSine
 * (fdtdrav.h:1486-1520) and the injection in calc_e (fdtdrav.h:726-733). Several sources may
 * be added; their edges may not overlap. Steps past n_samples inject zero. */
int fdtd_add_lumped_source(fdtd_handle* h, int32_t axis, const int32_t box[6], float resistance,
                           const float* voltage, int64_t n_samples, int32_t* id_out);
/* Lumped resistor on the same kind of edge box (defineResistor, fdtdrav.h:1429-1483). */
int fdtd_add_resistor(fdtd_handle* h, int32_t axis, const int32_t box[6], float resistance);

/* Zero-thickness conducting plate normal to `normal_axis` (0 x, 1 y, 2 z) at the box's low
 * coordinate on that axis: the sigma_e of the E edges it covers becomes sigma_1 / sigma_2 for its
 * two tangential components in axis order (x plate: y, z; y plate: x, z; z plate: x, y), after
 * the edge averages and before the update coefficients, later plates overriding earlier ones.
 * Covered edges, box = {is,js,ks,ie,je,ke}: x plate at i = is: Ey j in [js,je), k in [ks,ke];
 * Ez j in [js,je], k in [ks,ke). y plate at j = js: Ez i in [is,ie], k in [ks,ke); Ex i in
 * [is,ie), k in [ks,ke]. z plate at k = ks: Ex i in [is,ie), j in [js,je]; Ey i in [is,ie],
 * j in [js,je). Replaces definePlateX / definePlateY / definePlateZ (fdtdrav.h:1574-1679,
 * applied at fdtdrav.h:4162-4182). A plate may not cover the Ez edge of a lumped element, and
 * handles with plates take no design region and join no batch. */
int fdtd_add_plate(fdtd_handle* h, int32_t normal_axis, const int32_t box[6], float sigma_1, float sigma_2);
/* Zero-thickness sector plate in plane k = pz0: the Ex edges of nodes (i, j), i in [0, max_x),
 * j in [0, max_y], and the Ey edges of nodes i in [0, max_x], j in [0, max_y), whose position
 * (i dx, j dy) lies in the sector with apex (px1, py1), sides towards (px0, py0) and (px2, py2)
 * (node indices; tri = {px0, py0, px1, py1, px2, py2}) and radius `radius` (metres) take sigma_x /
 * sigma_y, like a plate (later plates and sectors override earlier ones). The test is the
 * reference's kernel's, with its roundings (nodes exactly on a side included or not as it does):
 * the point lies on the side of the third vertex of both sides and within the radius of the apex.
 * Replaces defineSec / tricheck (fdtdrav.h:1681-1744, 56-128). */
int fdtd_add_sector(fdtd_handle* h, const int32_t tri[6], int32_t pz0, float radius, int32_t max_x, int32_t max_y,
                    float sigma_x, float sigma_y);

/* Point probe of one field component at node (i,j,k): records, every step, the value right after
 * the component's main update and before its CPML correction, as sampleField does
 * (fdtdrav.h:234-246, called at 347, 372, 391, 740). Returns the probe's column in
 * fdtd_read_probes output. */
int fdtd_add_probe(fdtd_handle* h, int32_t component, int32_t i, int32_t j, int32_t k, int32_t* id_out);
/* Number of steps the device probe ring buffer keeps (default 4096). */
int fdtd_set_probe_capacity(fdtd_handle* h, int64_t steps);

/* Build the device tables (CPML profiles, per-material coefficients, lumped-edge coefficients):
 * replaces setCoefficients, setABCPML, defineSourceZ and defineResistor (fdtdrav.h:1223-1308,
 * 1747-2160, 1368-1483). Called implicitly by the first fdtd_step. */
int fdtd_prepare(fdtd_handle* h);

/* Advance n time steps: per step the E update (with source injection) then the H update, with
 * the CPML corrections and probe sampling fused in. Replaces the time loop of marchingLoop
 * (fdtdrav.h:4320-4355) and solver (fdtdrav.h:3188-3422). Stream-ordered, does not synchronise. */
int fdtd_step(fdtd_handle* h, int64_t n);
int fdtd_synchronize(fdtd_handle* h);
int64_t fdtd_current_step(const fdtd_handle* h);

/* Probe values of steps [first_step, first_step+n_steps) into out[n_steps][n_probes]
 * (host memory). FDTD_ERR_RANGE if some of those steps left the ring buffer. */
int fdtd_read_probes(fdtd_handle* h, int64_t first_step, int64_t n_steps, float* out);
int32_t fdtd_probe_count(const fdtd_handle* h);

/* Whole-field copies between the simulation and host memory (nz*ny*nx floats) or device memory
 * (dense nz*ny*nx floats, caller-owned). */
int fdtd_get_field(fdtd_handle* h, int32_t component, float* host_out);
int fdtd_set_field(fdtd_handle* h, int32_t component, const float* host_in);
int fdtd_get_field_device(fdtd_handle* h, int32_t component, float* dev_out);
int fdtd_set_field_device(fdtd_handle* h, int32_t component, const float* dev_in);

/* Checkpoint / resume of the full dynamic state (fields, CPML memory, step counter). The
 * reference has none. fdtd_state_bytes gives the size of the device buffer fdtd_save_state
 * writes (device memory, caller-owned). */
int64_t fdtd_state_bytes(const fdtd_handle* h);
int fdtd_save_state(fdtd_handle* h, void* dev_buf);
int fdtd_load_state(fdtd_handle* h, const void* dev_buf);

/* CPML grading (replaces setABCPML's sigma_max, fdtdrav.h:1794-1812). r0 = 0, the default: the
 * reference's sigma_opt = (m + 1) / (150 pi delta) times 1.5, the same for every slab thickness (the
 * reference has no reflection-coefficient parameter). 0 < r0 < 1: sigma_max of each slab from its
 * reflection coefficient at normal incidence, -(m + 1) ln(r0) / (2 eta0 P delta) with
 * eta0 = sqrt(mu0 / eps0), P the slab's cells and delta the axis' cell size (Gedney's polynomial
 * grading). The grading order m = 3, kappa_max = 5 and the linear alpha profile stay the
 * reference's. Takes effect at the next preparation or step; the CPML memory is kept. */
int fdtd_set_cpml_grading(fdtd_handle* h, float r0);

/* One 1-D CPML profile of an axis (0 = x, 1 = y, 2 = z) into host memory (n_axis floats):
 * kind 0 = b_e, 1 = a_e, 2 = b_m, 3 = a_m, 4 = kappa_e, 5 = kappa_m. These are the d_cpml_b/a
 * arrays and the kappa values that setABCPML computes (fdtdrav.h:1863-1906); nodes outside the
 * CPML hold b = a = 1.2e-38 and kappa = 1. Builds the tables if needed. */
int fdtd_get_cpml_profile(fdtd_handle* h, int32_t axis, int32_t kind, float* host_out);

/* Bytes of device memory the handle holds. */
int64_t fdtd_device_bytes(const fdtd_handle* h);

/* Port voltage and current. Registers the point probes of a port: the Ez samples of the voltage
 * box that voltMgpu sums for voltage_axis 0 / 1 / 2 (x / y / z, its direction 1 / 2 / 3; the
 * reference samples Ez for every direction, sampleField in calc_e fdtdrav.h:740, and only the
 * ranges and the scale change, fdtdrav.h:2214-2290):
 *   x: i in [is,ie), j in [js,je], k in [ks,ke];  y: i in [is,ie], j in [js,je), k in [ks,ke];
 *   z: i in [is,ie], j in [js,je], k in [ks,ke)
 * (k outer, then j, then i), and the current loop of currMgpu around the current box for
 * current_axis 0 / 1 / 2 (x / y / z, fdtdrav.h:2318-2480, cases 1 / 2 / 3):
 *   x: Hy(ie-1, j, ks-1), Hz(ie-1, je, k), Hy(ie-1, j, ke), Hz(ie-1, js-1, k)
 *   y: Hz(is-1, je-1, k), Hx(i, je-1, ke), Hz(ie, je-1, k), Hx(i, je-1, ks-1)
 *   z: Hy(ie, j, ke-1), Hx(i, js-1, ke-1), Hy(is-1, j, ke-1), Hx(i, je, ke-1)
 * for i in [is,ie], j in [js,je], k in [ks,ke] of the current box. Replaces the voltage / current
 * sample boxes of sampleField and the reductions voltMgpu / currMgpu (fdtdrav.h:2185-2488). Add
 * ports before the first step; their probes also appear as columns of fdtd_read_probes. */
int fdtd_add_port(fdtd_handle* h, int32_t voltage_axis, const int32_t voltage_box[6], int32_t current_axis,
                  const int32_t current_box[6], int32_t* id_out);
/* V(t) = csuf * sum of the voltage samples, csuf = -dx / ((je-js+1)(ke-ks+1)) (x),
 * -dy / ((ke-ks+1)(ie-is+1)) (y), -dz / ((ie-is+1)(je-js+1)) (z), and I(t) = a1 s1 + a2 s2 - a1 s3 - a2 s4
 * over the four probe groups above in order (a1, a2 = dy, dz for x; dz, dx for y; dy, dx for z)
 * for steps [first_step, first_step+n_steps), summed in the reference's order (host memory;
 * voltMgpu / currMgpu, fdtdrav.h:2185-2488). With time_average
 * set, I(t) becomes (I(t) + I(t+1)) / 2 over the window from the unaveraged I(t+1), and the last
 * step (I(t) + I'(t-1)) / 2 from the averaged I'(t-1), as the reference's in-place correcI produces
 * them (fdtdrav.h:2490-2508, called by calcVoltCurrent, fdtdrav.h:3129-3186). */
int fdtd_read_port(fdtd_handle* h, int32_t id, int64_t first_step, int64_t n_steps, int32_t time_average,
                   float* voltage, float* current);
/* Frequency response of a port over steps [first_step, first_step+n_steps): real-to-complex FFTs
 * (cuFFT, n_steps/2+1 bins, unnormalised) of V(t) and the time-averaged I(t), then per bin
 * a = (V + z0 I) / (2 sqrt(Re z0)), b = (V - z0 I) / (2 sqrt(Re z0)), s11 = b / a and
 * zin = z0 (1 + s11) / (1 - s11). Outputs are host arrays of n_steps/2+1 interleaved complex
 * floats; any may be NULL. Bin f is the frequency f / (n_steps dt). Replaces calc_otm / calc_otm2
 * (fdtdrav.h:2988-3127) and c_zinS11 (fdtdrav.h:2510-2548). Synchronises the handle's stream. */
int fdtd_port_spectrum(fdtd_handle* h, int32_t id, int64_t first_step, int64_t n_steps, float z0_re, float z0_im,
                       float* v_spectrum, float* i_spectrum, float* s11, float* zin);
/* The per-bin step of fdtd_port_spectrum on spectra the caller already holds (host arrays of
 * n_bins interleaved complex floats): s11 and zin for reference impedance z0, on the current
 * device's default stream. Replaces c_zinS11 (fdtdrav.h:2510-2548) as calc_otm2 uses it on
 * precomputed spectra (fdtdrav.h:3054-3127). */
int fdtd_port_zin(int64_t n_bins, const float* v_spectrum, const float* i_spectrum, float z0_re, float z0_im,
                  float* s11, float* zin);

/* ---- The reference's whole run ------------------------------------------------------------ */

/* Source waveform of setGauss / setSine (fdtdrav.h:1486-1520), evaluated on the current device so
 * that expf / sinf are CUDA's: type 1 out[m] = amp exp(-((m dt - t_0)^2) / tau^2), type 3
 * out[m] = amp sin(2 pi freq dt m), type 2 zero (the reference leaves that signal unset).
 * n values to host memory. */
int fdtd_source_waveform(int32_t type, float amp, float freq, float dt, float t_0, float tau, float pi, int64_t n,
                         float* out);

/* marchingLoop (fdtdrav.h:3425-4387) with its parameter list, plus the host arrays voltage and
 * current (n_t_steps floats each) that receive V(t) and the time-averaged I(t) which the reference
 * computes in calcVoltCurrent and writes to its result files. Geometry in metres is converted to
 * node indices as the reference does (calc_index, offsets of CPML and air buffer, NZ rounded up to
 * a multiple of NUMDEV); the whole domain then runs on the current device. Bricks (with their
 * per-axis values, fdtd_set_materials_axes), z plates (pec_*), the z-directed lumped source with its waveform
 * (source_tp 1 Gaussian, 3 sine, 2 none), the resistor (z edges, as defineResistor) and the port
 * (voltage direction 3, current direction 1 / 2 / 3). c and nc are unused, as in the reference. */
int fdtd_marching_loop(
    const int NUMDEV, float eps_0, float pi, float mu_0, float c, float dx, float dy, float dz, float dt, int X, int Y,
    int Z, int n_t_steps, int pml_x_n, int pml_y_n, int pml_z_n, int pml_x_p, int pml_y_p, int pml_z_p, int air_buff_x_n,
    int air_buff_y_n, int air_buff_z_n, int air_buff_x_p, int air_buff_y_p, int air_buff_z_p, int source_tp,
    float source_freq, float source_amp, float source_min_x, float source_min_y, float source_min_z, float source_max_x,
    float source_max_y, float source_max_z, int source_direction, float rs, float nc, float tau, float t_0,
    const float* brick_min_x, const float* brick_min_y, const float* brick_min_z, const float* brick_max_x,
    const float* brick_max_y, const float* brick_max_z, const float* brick_sigma_e_x, const float* brick_sigma_e_y,
    const float* brick_sigma_e_z, const float* brick_eps_r_x, const float* brick_eps_r_y, const float* brick_eps_r_z,
    const float* brick_sigma_m_x, const float* brick_sigma_m_y, const float* brick_sigma_m_z, const float* brick_mu_r_x,
    const float* brick_mu_r_y, const float* brick_mu_r_z, int brick_opt, int brick_num, const float* pec_min_x,
    const float* pec_min_y, const float* pec_min_z, const float* pec_max_x, const float* pec_max_y,
    const float* pec_max_z, const float* pec_sigma_e_x, const float* pec_sigma_e_y, const float* pec_sigma_e_z,
    int pec_opt, int pec_num, float resistor_min_x, float resistor_min_y, float resistor_min_z, float resistor_max_x,
    float resistor_max_y, float resistor_max_z, float resistor_resist, int resistor_direction, int resistor_opt,
    float sampled_voltage_min_x, float sampled_voltage_min_y, float sampled_voltage_min_z, float sampled_voltage_max_x,
    float sampled_voltage_max_y, float sampled_voltage_max_z, int voltage_direction, float sampled_current_min_x,
    float sampled_current_min_y, float sampled_current_min_z, float sampled_current_max_x, float sampled_current_max_y,
    float sampled_current_max_z, int current_direction, float* voltage, float* current);

/* ---- Design region and adjoint gradient (no reference counterpart: the reference has no
 * gradient; its commented-out differential-evolution optimiser, fdtdrav.h:2758-2986, is the
 * gradient-free alternative it never finished). ---- */

/* Cells [box[0],box[3]) x [box[1],box[4]) x [box[2],box[5]) become the design region: eps_r per
 * cell from `eps_r` ((box[5]-box[2]) * (box[4]-box[1]) * (box[3]-box[0]) floats, x fastest),
 * sigma_e, mu_r and sigma_m from `base` (its eps_r is ignored). The cells get the reserved material
 * index 255 (so the table may hold at most 255 materials), painted over what they held. The E edges
 * of the region must be interior nodes (outside the CPML slabs and the boundary planes) and no
 * lumped element may touch it. Calling again with the same box only replaces eps_r. */
int fdtd_set_design_region(fdtd_handle* h, const int32_t box[6], const fdtd_material* base, const float* eps_r);

/* Figure of merit J = sum over the next n steps of dt * Ez(i,j,k)^2, Ez sampled after each step's E
 * update at an Ez edge outside the CPML. Runs the n steps and records what the backward needs:
 * checkpoint_every = K > 0 keeps the full state every K steps (the backward recomputes each segment
 * from its checkpoint, keeping only the design-region E); K = 0 keeps the design-region E of every
 * step instead (no recompute; (n+1) * 3 * (box+1)^3 floats). *J is the FP64 sum. */
int fdtd_adjoint_forward(fdtd_handle* h, int64_t n, int32_t checkpoint_every, int32_t i, int32_t j, int32_t k, double* J);

/* dJ/d(eps_r) of every design cell for the steps of the last fdtd_adjoint_forward, by the discrete
 * adjoint of the FP32 update (CPML memory and lumped elements included), accumulated in FP64 into
 * the host array `grad` (shaped like eps_r). The handle ends in the state the forward left. */
int fdtd_adjoint_backward(fdtd_handle* h, double* grad);

/* fdtd_adjoint_forward and fdtd_adjoint_backward of n distinct handles (each with its own design
 * region), every handle's work enqueued on its own stream before any is waited for, so that
 * handles run concurrently. probes holds n (i, j, k) triples, J n sums, grads n host arrays shaped
 * like each handle's eps_r. J and the gradients equal those of the per-handle calls bit for bit;
 * each handle ends in the state its forward left. */
int fdtd_batch_adjoint(fdtd_handle* const* handles, int32_t n, int64_t steps, int32_t checkpoint_every,
                       const int32_t* probes, double* J, double* const* grads);

/* ---- Batched launch (no reference counterpart: the reference runs one domain per process). A
 * batch advances many independent handles of any sizes together, its launches captured in CUDA
 * graphs, in one of three forms. Chains (cluster -1, the default): each instance runs its own
 * two-pass kernels on its own branch of the graph, every branch concurrent with the others. Flat
 * (cluster 0): per step one E kernel and one H kernel over the 32 x 8 blocks of every plane of
 * every instance, one node per thread. Persistent (cluster 1, 2, 4 or 8): one kernel for all
 * steps, each instance owned by a thread-block cluster for all of its steps (E update, cluster
 * barrier, H update, cluster barrier), instances taken longest first from a queue. Every instance
 * produces the bits fdtd_step would produce. ---- */
typedef struct fdtd_batch fdtd_batch;

/* A batch over n distinct handles on the current device (none with a design region). The handles
 * keep their state, tables and probe rings; between fdtd_batch_create and fdtd_batch_destroy they
 * may still be read, saved or stepped alone: every launch picks up each handle's current buffers
 * and step, after waiting for the handle's own stream. */
int fdtd_batch_create(fdtd_handle* const* handles, int32_t n, fdtd_batch** out);
int fdtd_batch_destroy(fdtd_batch* b);
/* Stream of the batch launches: a created stream, not the legacy default stream (the launch is
 * captured in a CUDA graph). By default the batch uses a stream of its own. */
int fdtd_batch_set_stream(fdtd_batch* b, void* stream);
/* Form and shape: cluster -1 = chains, 0 = flat (both 256 threads per CTA), or the persistent
 * form's cluster size (1, 2, 4 or 8 CTAs per instance) with its CTA size (128, 256 or 512). */
int fdtd_batch_set_config(fdtd_batch* b, int32_t cluster, int32_t threads);
int fdtd_batch_get_config(const fdtd_batch* b, int32_t* cluster, int32_t* threads, int32_t* n_clusters);
/* Autotuner: times `steps` steps of the whole batch in the chain and flat forms and for every
 * cluster and CTA size of the persistent form (a first untimed run captures each candidate's
 * graphs), restores every instance's state after each run, keeps the fastest (its time in
 * *best_ms if not NULL). */
int fdtd_batch_tune(fdtd_batch* b, int64_t steps, double* best_ms);
/* Advance every instance by `steps` steps (graph launches, asynchronous on the batch stream). */
int fdtd_batch_step(fdtd_batch* b, int64_t steps);
/* Wait for the batch stream; FDTD_ERR_DEVICE if an instance's kernel reported an error. */
int fdtd_batch_synchronize(fdtd_batch* b);

/* Maximum bytes of FDTD_STEP_STATIC_SCRATCH: one second field set, one second CPML memory set and
 * the sweep's work list. Enough for a 64^3 grid with 10-cell CPML on all faces (about 9.8 MiB). */
#define FDTD_STEP_STATIC_SCRATCH_BYTES (16u << 20)

/* No reference counterpart. Advances n steps with the fused sweep like fdtd_step under
 * FDTD_SCHEDULE_FUSED, with bit-identical fields, CPML memory and probe samples. This call
 * allocates no device memory. fdtd_step allocates a second field set and CPML set (plus the
 * sweep's work list) the first time it runs the fused sweep. The ping-pong target here is instead
 * a fixed static device array of FDTD_STEP_STATIC_SCRATCH_BYTES inside the library.
 * It is for callers that cannot allocate while stepping: callers whose device memory is reserved
 * in full up front (by their own pool) so that a lazy allocation would fail, and callers that must
 * not let a step call synchronise the device (cudaMalloc / cudaFree may).
 *  - The handle must be prepared (fdtd_prepare after the last change to materials, lumped elements
 *    or probes), because preparation allocates; otherwise FDTD_ERR_STATE. The calling thread's
 *    current device must be the handle's device.
 *  - Grids whose scratch exceeds FDTD_STEP_STATIC_SCRATCH_BYTES are rejected with
 *    FDTD_ERR_RANGE, and the message gives the bytes needed.
 *  - The first call on each device looks up the array's address (cudaGetSymbolAddress) and sets
 *    the sweep kernels' shared-memory limit; these are not stream operations. A call with n = 0
 *    does only this set-up; make it once per device before a section that must issue nothing
 *    but stream work. The address is kept for the life of the process: after a cudaDeviceReset
 *    it is stale, so do not use this call across a device reset.
 *  - Each call uploads the sweep's work list (planned once per handle into pinned host memory)
 *    into the scratch with one asynchronous host-to-device copy on the handle's stream.
 *  - Nothing in the scratch needs to start at zero or to survive between calls: with an odd n the
 *    call first copies the handle's CPML memory into it, every scratch element a step reads was
 *    written earlier in the same call, and the result is back in the handle's own buffers when
 *    the call's stream work completes.
 *  - The scratch is one per device and per process. Calls whose stream work overlaps on the device
 *    (other handles, other streams, other threads) race on it and corrupt each other's results;
 *    order them (one stream, or events), as with any shared buffer. */
int fdtd_step_static_scratch(fdtd_handle* h, int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* FDTD_API_H */
