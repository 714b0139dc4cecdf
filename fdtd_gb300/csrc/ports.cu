// Port spectra: the frequency-domain post-processing of a port's V(t) and I(t).
//
// Follows calc_otm / calc_otm2 (fdtdrav.h:2988-3051, 3054-3127) and c_zinS11 (fdtdrav.h:2510-2548):
// real-to-complex FFTs of V(t) and the time-averaged I(t) (n_t_steps / 2 + 1 bins, unnormalised),
// then per bin a = (V + z0 I) / (2 sqrt(Re z0)), b = (V - z0 I) / (2 sqrt(Re z0)), s11 = b / a and
// zin = z0 (1 + s11) / (1 - s11), with cuComplex.h's complex arithmetic as the reference uses it.
//
// The two transforms run as one batched cuFFT plan over a [2][n] array (V row, I row). The
// reference plans a batch of 2 but executes it on each signal separately (reading and writing past
// the ends of its one-signal buffers); the batch here is the one the plan describes.
#include <cuComplex.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <string>

#include "fdtd_api.h"
#include "ports.h"

namespace fdtd {

namespace {

__global__ void k_port_zin(const cuFloatComplex* __restrict__ spec, int nf, cuFloatComplex z0,
                           cuFloatComplex* __restrict__ s11, cuFloatComplex* __restrict__ zin) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const cuFloatComplex v = spec[f], i = spec[nf + f];
    const cuFloatComplex scale = make_cuFloatComplex(2.f * sqrtf(cuCrealf(z0)), 0.f);
    const cuFloatComplex zi = cuCmulf(z0, i);
    const cuFloatComplex a = cuCdivf(cuCaddf(v, zi), scale);
    const cuFloatComplex b = cuCdivf(cuCsubf(v, zi), scale);
    const cuFloatComplex s = cuCdivf(b, a);
    const cuFloatComplex one = make_cuFloatComplex(1.f, 0.f);
    s11[f] = s;
    zin[f] = cuCmulf(z0, cuCdivf(cuCaddf(one, s), cuCsubf(one, s)));
}

struct Scratch {
    void* p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace

int port_zin(cudaStream_t st, int nf, const float* v_spec, const float* i_spec, float z0_re, float z0_im,
             float* s11_out, float* zin_out, std::string* err) {
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        *err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FDTD_ERR_OOM : FDTD_ERR_CUDA;
    };
    const size_t bin_bytes = (size_t)nf * sizeof(cuFloatComplex);
    Scratch buf;
    cudaError_t e = cudaMalloc(&buf.p, 4 * bin_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc port zin");
    cuFloatComplex* d_spec = (cuFloatComplex*)buf.p;
    cuFloatComplex* d_s11 = d_spec + 2 * nf;
    cuFloatComplex* d_zin = d_s11 + nf;
    if ((e = cudaMemcpyAsync(d_spec, v_spec, bin_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_spec + nf, i_spec, bin_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(e, "port spectra H2D");
    k_port_zin<<<(nf + 255) / 256, 256, 0, st>>>(d_spec, nf, make_cuFloatComplex(z0_re, z0_im), d_s11, d_zin);
    e = cudaGetLastError();
    if (e == cudaSuccess && s11_out) e = cudaMemcpyAsync(s11_out, d_s11, bin_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && zin_out) e = cudaMemcpyAsync(zin_out, d_zin, bin_bytes, cudaMemcpyDeviceToHost, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "port zin");
    if (es != cudaSuccess) return cuda_fail(es, "port zin sync");
    return FDTD_OK;
}

int port_spectra(cudaStream_t st, int n, const float* volt, const float* curr, float z0_re, float z0_im,
                 float* v_out, float* i_out, float* s11_out, float* zin_out, std::string* err) {
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        *err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FDTD_ERR_OOM : FDTD_ERR_CUDA;
    };
    const int nf = n / 2 + 1;
    const size_t sig_bytes = (size_t)n * sizeof(float), bin_bytes = (size_t)nf * sizeof(cuFloatComplex);
    // [2][n] signals, [2][nf] spectra, [nf] s11, [nf] zin; every part starts on a 16-byte boundary
    const size_t sig_part = (2 * sig_bytes + 15) / 16 * 16;
    Scratch buf;
    cudaError_t e = cudaMalloc(&buf.p, sig_part + 4 * bin_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc port spectra");
    float* d_sig = (float*)buf.p;
    cuFloatComplex* d_spec = (cuFloatComplex*)((char*)buf.p + sig_part);
    cuFloatComplex* d_s11 = d_spec + 2 * nf;
    cuFloatComplex* d_zin = d_s11 + nf;
    if ((e = cudaMemcpyAsync(d_sig, volt, sig_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_sig + n, curr, sig_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(e, "port signals H2D");
    cufftHandle plan;
    int dims[1] = {n};
    cufftResult r = cufftPlanMany(&plan, 1, dims, nullptr, 1, n, nullptr, 1, nf, CUFFT_R2C, 2);
    if (r != CUFFT_SUCCESS) {
        *err = "cufftPlanMany failed (" + std::to_string((int)r) + ")";
        return FDTD_ERR_CUDA;
    }
    r = cufftSetStream(plan, st);
    if (r == CUFFT_SUCCESS) r = cufftExecR2C(plan, d_sig, d_spec);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(plan);
        *err = "cufftExecR2C failed (" + std::to_string((int)r) + ")";
        return FDTD_ERR_CUDA;
    }
    k_port_zin<<<(nf + 255) / 256, 256, 0, st>>>(d_spec, nf, make_cuFloatComplex(z0_re, z0_im), d_s11, d_zin);
    e = cudaGetLastError();
    if (e == cudaSuccess && v_out) e = cudaMemcpyAsync(v_out, d_spec, bin_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && i_out) e = cudaMemcpyAsync(i_out, d_spec + nf, bin_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && s11_out) e = cudaMemcpyAsync(s11_out, d_s11, bin_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && zin_out) e = cudaMemcpyAsync(zin_out, d_zin, bin_bytes, cudaMemcpyDeviceToHost, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    cufftDestroy(plan);
    if (e != cudaSuccess) return cuda_fail(e, "port spectra");
    if (es != cudaSuccess) return cuda_fail(es, "port spectra sync");
    return FDTD_OK;
}

}  // namespace fdtd
