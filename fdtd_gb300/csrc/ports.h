// Port spectra (calc_otm / c_zinS11 of the reference) on the device.
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace fdtd {

// V(t), I(t): n host floats each. Outputs (host, n/2+1 interleaved complex each, any may be NULL):
// the spectra of V and I, s11 and zin for the complex reference impedance z0. Synchronises `st`.
// Returns FDTD_OK, or FDTD_ERR_CUDA / FDTD_ERR_OOM with the message in *err.
int port_spectra(cudaStream_t st, int n, const float* volt, const float* curr, float z0_re, float z0_im,
                 float* v_out, float* i_out, float* s11_out, float* zin_out, std::string* err);

// s11 and zin of given spectra (n_bins interleaved complex each, host), as port_spectra does after
// its transforms. Synchronises `st`.
int port_zin(cudaStream_t st, int n_bins, const float* v_spec, const float* i_spec, float z0_re, float z0_im,
             float* s11_out, float* zin_out, std::string* err);

}  // namespace fdtd
