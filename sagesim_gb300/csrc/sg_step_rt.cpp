// sg_step_rt.cpp -- NVRTC runtime for compiled step functions.
#include "sg_step_rt.h"

#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sagesim_gb300.h"
#include "sg_embedded_headers.h" // generated at build time: kSgPhiloxHeader, kSgStepHeader

struct SgCompiledStep {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
};

namespace {

struct NvrtcApi {
    bool loaded = false;
    std::string error;
    const char *(*GetErrorString)(nvrtcResult) = nullptr;
    nvrtcResult (*CreateProgram)(nvrtcProgram *, const char *, const char *, int, const char *const *,
                                 const char *const *) = nullptr;
    nvrtcResult (*CompileProgram)(nvrtcProgram, int, const char *const *) = nullptr;
    nvrtcResult (*GetCUBINSize)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*GetCUBIN)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*GetProgramLogSize)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*GetProgramLog)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*DestroyProgram)(nvrtcProgram *) = nullptr;
};

NvrtcApi &nvrtc()
{
    static NvrtcApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/lib64/libnvrtc.so"};
        void *h = nullptr;
        for (const char *nm : names) {
            h = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
            if (h) break;
        }
        if (!h) {
            api.error = "cannot load libnvrtc (dlopen failed)";
            return;
        }
#define SG_SYM(field, sym)                                                                     \
    api.field = reinterpret_cast<decltype(api.field)>(dlsym(h, sym));                          \
    if (!api.field) {                                                                          \
        api.error = std::string("libnvrtc lacks ") + sym;                                      \
        return;                                                                                \
    }
        SG_SYM(GetErrorString, "nvrtcGetErrorString");
        SG_SYM(CreateProgram, "nvrtcCreateProgram");
        SG_SYM(CompileProgram, "nvrtcCompileProgram");
        SG_SYM(GetCUBINSize, "nvrtcGetCUBINSize");
        SG_SYM(GetCUBIN, "nvrtcGetCUBIN");
        SG_SYM(GetProgramLogSize, "nvrtcGetProgramLogSize");
        SG_SYM(GetProgramLog, "nvrtcGetProgramLog");
        SG_SYM(DestroyProgram, "nvrtcDestroyProgram");
#undef SG_SYM
        api.loaded = true;
    });
    return api;
}

bool valid_identifier(const char *s)
{
    if (!s || !*s) return false;
    for (const char *p = s; *p; ++p) {
        const char c = *p;
        const bool ok = (c == '_') || (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') ||
                        (p != s && c >= '0' && c <= '9');
        if (!ok) return false;
    }
    return true;
}

} // namespace

std::string sg_step_rt_source(const char *src, const char *entry)
{
    std::string s;
    s += kSgPhiloxHeader;
    s += "\n";
    s += kSgStepHeader;
    s += "\n// ---- user step ----\n";
    s += src;
    s += "\n// ---- tile-walking wrapper ----\n";
    s += "extern \"C\" __global__ void __launch_bounds__(256) sg_compiled_step(sg_step_args a)\n"
         "{\n"
         "    sg_ctx ctx;\n"
         "    ctx.tick = a.tick0 + a.r;\n"
         "    ctx.key = a.key;\n"
         "    ctx.c0b = sg_c0base(ctx.tick);\n"
         "    ctx.r = a.r;\n"
         "    ctx.lids = a.lids;\n"
         "    ctx.off = a.off;\n"
         "    ctx.idx = a.idx;\n"
         "    ctx.g = a.g;\n"
         "    ctx.props = a.props;\n"
         "    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {\n"
         "        const int b = a.tiles[4 * t + 1], e = a.tiles[4 * t + 2];\n"
         "        for (int i = b + (int)threadIdx.x; i < e; i += (int)blockDim.x) ";
    s += entry;
    s += "(ctx, i);\n"
         "    }\n"
         "}\n";
    return s;
}

int sg_step_rt_compile(int device, const char *src, const char *entry, SgCompiledStep **out,
                       std::string *log)
{
    *out = nullptr;
    if (!valid_identifier(entry)) {
        *log = "entry must be a C identifier";
        return SG_ERR_INVALID;
    }
    NvrtcApi &api = nvrtc();
    if (!api.loaded) {
        *log = api.error;
        return SG_ERR_COMPILE;
    }
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    char arch[64];
    // "a" = architecture-specific features (sm_103a on GB300)
    snprintf(arch, sizeof arch, "--gpu-architecture=sm_%d%da", major, minor);
    const std::string full = sg_step_rt_source(src, entry);
    nvrtcProgram prog = nullptr;
    nvrtcResult r = api.CreateProgram(&prog, full.c_str(), "sg_step.cu", 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) {
        *log = std::string("nvrtcCreateProgram: ") + api.GetErrorString(r);
        return SG_ERR_COMPILE;
    }
    const char *opts[] = {arch, "--std=c++17", "-default-device", "--fmad=false", "-lineinfo"};
    r = api.CompileProgram(prog, 5, opts);
    size_t logsz = 0;
    api.GetProgramLogSize(prog, &logsz);
    std::string lg(logsz, '\0');
    if (logsz) api.GetProgramLog(prog, &lg[0]);
    if (r != NVRTC_SUCCESS) {
        *log = std::string("NVRTC: ") + api.GetErrorString(r) + "\n" + lg;
        api.DestroyProgram(&prog);
        return SG_ERR_COMPILE;
    }
    size_t cubsz = 0;
    api.GetCUBINSize(prog, &cubsz);
    std::vector<char> cubin(cubsz);
    api.GetCUBIN(prog, cubin.data());
    api.DestroyProgram(&prog);

    auto *cs = new SgCompiledStep();
    cudaError_t ce = cudaLibraryLoadData(&cs->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        *log = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
        delete cs;
        return SG_ERR_CUDA;
    }
    ce = cudaLibraryGetKernel(&cs->kernel, cs->lib, "sg_compiled_step");
    if (ce != cudaSuccess) {
        *log = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(ce);
        cudaLibraryUnload(cs->lib);
        delete cs;
        return SG_ERR_CUDA;
    }
    *out = cs;
    return SG_OK;
}

cudaError_t sg_step_rt_launch(SgCompiledStep *s, const sg_step_args &a, int grid, cudaStream_t st)
{
    sg_step_args copy = a;
    void *args[] = {&copy};
    return cudaLaunchKernel((const void *)s->kernel, dim3(grid), dim3(256), args, 0, st);
}

void sg_step_rt_destroy(SgCompiledStep *s)
{
    if (!s) return;
    if (s->lib) cudaLibraryUnload(s->lib);
    delete s;
}
