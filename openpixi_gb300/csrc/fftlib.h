// fftlib.h -- cuFFT loaded at run time, so that the library itself does not
// depend on libcufft (its users fail with a status code when it is absent).
#pragma once
#include <dlfcn.h>

#include <string>

#include <cufft.h>

namespace opx {

struct FFTLib {
    void *h = nullptr;
    decltype(&cufftPlanMany) planMany = nullptr;
    decltype(&cufftExecZ2Z) execZ2Z = nullptr;
    decltype(&cufftSetStream) setStream = nullptr;
    decltype(&cufftDestroy) destroy = nullptr;
    bool load(std::string &err) {
        if (h) return true;
        const char *names[] = {"libcufft.so.12", "libcufft.so", "/usr/local/cuda/lib64/libcufft.so.12"};
        for (const char *n : names) {
            h = dlopen(n, RTLD_NOW | RTLD_LOCAL);
            if (h) break;
        }
        if (!h) { err = "cuFFT library not found (libcufft.so.12)"; return false; }
        planMany = (decltype(planMany))dlsym(h, "cufftPlanMany");
        execZ2Z = (decltype(execZ2Z))dlsym(h, "cufftExecZ2Z");
        setStream = (decltype(setStream))dlsym(h, "cufftSetStream");
        destroy = (decltype(destroy))dlsym(h, "cufftDestroy");
        if (!planMany || !execZ2Z || !setStream || !destroy) { err = "cuFFT symbols missing"; h = nullptr; return false; }
        return true;
    }
};
// one loader per process
inline FFTLib &fft_lib() {
    static FFTLib lib;
    return lib;
}

// An owned cuFFT plan.
struct FFTPlan {
    cufftHandle h = 0;
    bool ok = false;
    FFTPlan() = default;
    FFTPlan(const FFTPlan &) = delete;
    FFTPlan &operator=(const FFTPlan &) = delete;
    ~FFTPlan() { if (ok) fft_lib().destroy(h); }
    // rank-dimensional complex-to-complex transforms, batch of `batch` contiguous arrays
    bool make(int rank, int *dims, int batch, cudaStream_t st) {
        FFTLib &L = fft_lib();
        ok = L.planMany(&h, rank, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_Z2Z, batch) == CUFFT_SUCCESS;
        if (ok) L.setStream(h, st);
        return ok;
    }
};

}  // namespace opx
