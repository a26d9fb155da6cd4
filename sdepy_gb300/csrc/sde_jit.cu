// Runtime compilation of user SDE programs (sdepy's integrate decorator,
// sdepy/integration.py:1843-1955).
//
// The straight-line program of an SdeUserProgram is written out as CUDA C++
// (UserJitFn<R>::coefs: one statement per instruction, the interpreter's own
// arithmetic -- Ar<R> / UFn<R> / np_max -- so FP64 results are bit-identical
// to user_coefs), compiled with NVRTC for sm_103a together with the forward
// kernel header, and the resulting cubin is loaded through the runtime's
// library API.  The forward kernel instantiated with SDE_MODEL_USER_JIT /
// SDE_MODEL_USER_SYS_JIT then evaluates the coefficients inline, with no
// register file in local memory and no dispatch; the adjoint kernel
// (sde_adj_user.cuh) also gets the program's reverse-mode step
// (UserJitAdj<R>::back), generated here instruction by instruction.
// Kernels are cached per generated source (program, precision, group
// width, noise mode, forward or adjoint) for the life of the process; with
// SDEPY_GB300_JIT_DUMP set to a directory, each generated source is also
// written there (sde_jit_<hash>.cu) for inspection.
//
// NVRTC is loaded with dlopen: a library without it still runs the
// interpreted kernels (SdeUserProgram.jit = 0).
#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "sde_jit.h"
#include "sde_kernels.cuh"

namespace sdegpu {

namespace {

struct Nvrtc {
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcAddNameExpression) add_name = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetLoweredName) lowered = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
    bool ok = false;
    std::string include_dir;   // csrc/, beside the library's _native/
};

Nvrtc &nvrtc() {
    static Nvrtc N;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/lib64/libnvrtc.so"};
        void *h = nullptr;
        for (const char *n : names)
            if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) return;
#define SDE_NVRTC(field, sym) N.field = (decltype(N.field))dlsym(h, #sym)
        SDE_NVRTC(create, nvrtcCreateProgram);
        SDE_NVRTC(add_name, nvrtcAddNameExpression);
        SDE_NVRTC(compile, nvrtcCompileProgram);
        SDE_NVRTC(log_size, nvrtcGetProgramLogSize);
        SDE_NVRTC(log, nvrtcGetProgramLog);
        SDE_NVRTC(lowered, nvrtcGetLoweredName);
        SDE_NVRTC(cubin_size, nvrtcGetCUBINSize);
        SDE_NVRTC(cubin, nvrtcGetCUBIN);
        SDE_NVRTC(destroy, nvrtcDestroyProgram);
#undef SDE_NVRTC
        Dl_info info;
        if (!dladdr((void *)&sde_jit_available, &info) || !info.dli_fname) return;
        std::string so = info.dli_fname;   // .../sdepy_gb300/_native/libsdepy_gb300.so
        size_t a = so.rfind('/');
        if (a == std::string::npos) return;
        size_t b = so.rfind('/', a - 1);
        if (b == std::string::npos) return;
        N.include_dir = so.substr(0, b) + "/csrc";
        N.ok = N.create && N.add_name && N.compile && N.log_size && N.log && N.lowered && N.cubin_size &&
               N.cubin && N.destroy;
    });
    return N;
}

// one instruction of the program as a statement on r[]
std::string op_statement(const SdeUserProgram &u, uint32_t op) {
    const int code = op & 0xff, d = (op >> 8) & 0xff, ia = (op >> 16) & 0xff, ib = op >> 24;
    char buf[160];
    const char *un = nullptr, *bin = nullptr;
    switch (code) {
    case SDE_UOP_CONST: {
        uint64_t bits;
        memcpy(&bits, &u.consts[ia], sizeof bits);
        snprintf(buf, sizeof buf, "r[%d] = (R)__longlong_as_double((long long)0x%016llxULL);", d,
                 (unsigned long long)bits);
        return buf;
    }
    case SDE_UOP_ADD: bin = "A::add"; break;
    case SDE_UOP_SUB: bin = "A::sub"; break;
    case SDE_UOP_MUL: bin = "A::mul"; break;
    case SDE_UOP_MAX: bin = "np_max"; break;
    case SDE_UOP_MIN: bin = "np_min"; break;
    case SDE_UOP_POW: bin = "F::pow_"; break;
    case SDE_UOP_DIV:
        snprintf(buf, sizeof buf, "r[%d] = r[%d] / r[%d];", d, ia, ib);
        return buf;
    case SDE_UOP_NEG: snprintf(buf, sizeof buf, "r[%d] = -r[%d];", d, ia); return buf;
    case SDE_UOP_ABS: un = "fabs"; break;
    case SDE_UOP_EXP: un = "F::exp_"; break;
    case SDE_UOP_LOG: un = "F::log_"; break;
    case SDE_UOP_SQRT: un = "A::sqrt_"; break;
    case SDE_UOP_SIN: un = "F::sin_"; break;
    case SDE_UOP_COS: un = "F::cos_"; break;
    case SDE_UOP_TAN: un = "F::tan_"; break;
    case SDE_UOP_TANH: un = "F::tanh_"; break;
    case SDE_UOP_EXPM1: un = "F::expm1_"; break;
    case SDE_UOP_LOG1P: un = "F::log1p_"; break;
    case SDE_UOP_ARCTAN: un = "F::atan_"; break;
    default: snprintf(buf, sizeof buf, "r[%d] = r[%d];", d, ia); return buf;   // SDE_UOP_COPY
    }
    if (bin) snprintf(buf, sizeof buf, "r[%d] = %s(r[%d], r[%d]);", d, bin, ia, ib);
    else snprintf(buf, sizeof buf, "r[%d] = %s(r[%d]);", d, un, ia);
    return buf;
}

std::string kernel_name(const char *rt, int model, int maxm, bool inject, bool jumps) {
    char buf[160];
    snprintf(buf, sizeof buf, "sdegpu::sde_fwd_kernel<%s, %d, %d, %s, %s, false, false>", rt, model, maxm,
             inject ? "true" : "false", jumps ? "true" : "false");
    return buf;
}

// the sources of a program's terms as a constexpr function of the term index
std::string src_function(const SdeUserProgram &u) {
    std::string s = "  static __device__ __forceinline__ constexpr int src(int i) { return ";
    for (int i = 0; i < u.n_terms; ++i)
        s += "i == " + std::to_string(i) + " ? " + std::to_string(u.term_source[i]) + " : ";
    return s + "-1; }\n";
}

// UserJitFn<R>: the program's shape as constants (NEQ equations, NT terms,
// src(i) the source of term i) and the program as straight-line
// coefficient code
std::string coefs_struct(const SdeUserProgram &u, const char *rt) {
    std::string s = "template <> struct UserJitFn<";
    s += rt;
    s += "> {\n  typedef ";
    s += rt;
    s += " R;\n  static constexpr int NEQ = " + std::to_string(u.n_eq) + ", NT = " + std::to_string(u.n_terms) +
         ";\n" + src_function(u);
    s += "  static __device__ __forceinline__ void coefs(const R *xs, R t, const R (&p)[6],"
         " R (*out)[SDE_USER_MAX_TERMS]) {\n"
         "    typedef Ar<R> A;\n    typedef UFn<R> F;\n    R r[SDE_USER_MAX_REGS];\n"
         "    r[0] = xs[0];\n    r[1] = t;\n";
    for (int i = 0; i < 6; ++i) s += "    r[" + std::to_string(2 + i) + "] = p[" + std::to_string(i) + "];\n";
    for (int e = 1; e < u.n_eq; ++e) s += "    r[" + std::to_string(7 + e) + "] = xs[" + std::to_string(e) + "];\n";
    for (int i = 0; i < u.n_ops; ++i) s += "    " + op_statement(u, u.ops[i]) + "\n";
    for (int e = 0; e < u.n_eq; ++e)
        for (int j = 0; j < SDE_USER_MAX_TERMS; ++j)
            s += "    out[" + std::to_string(e) + "][" + std::to_string(j) + "] = " +
                 (j < u.n_terms ? "r[" + std::to_string(u.term_register[e][j]) + "]" : std::string("R(0)")) + ";\n";
    s += "  }\n};\n";
    return s;
}

std::string jit_source(const SdeUserProgram &u, const char *rt, int model, int maxm, bool inject, bool jumps) {
    return "#include \"sde_kernels.cuh\"\nnamespace sdegpu {\n" + coefs_struct(u, rt) + "template __global__ void " +
           kernel_name(rt, model, maxm, inject, jumps) + "(const __grid_constant__ FwdArgs<" + rt +
           ">);\n}  // namespace sdegpu\n";
}

// the parameters a program reads: 1 + the highest j of a register 2 + j
// read by an instruction or a term
int params_read(const SdeUserProgram &u) {
    int np = 0;
    auto see = [&](int r) {
        if (r >= 2 && r <= 7 && r - 1 > np) np = r - 1;
    };
    for (int i = 0; i < u.n_ops; ++i) {
        const uint32_t op = u.ops[i];
        const int code = op & 0xff;
        if (code == SDE_UOP_CONST) continue;
        see((op >> 16) & 0xff);
        if (code == SDE_UOP_ADD || code == SDE_UOP_SUB || code == SDE_UOP_MUL || code == SDE_UOP_DIV ||
            code == SDE_UOP_MAX || code == SDE_UOP_MIN || code == SDE_UOP_POW)
            see(op >> 24);
    }
    for (int e = 0; e < u.n_eq; ++e)
        for (int i = 0; i < u.n_terms; ++i) see(u.term_register[e][i]);
    return np;
}

// one instruction's reverse-mode statements: b[] holds the adjoints of the
// registers; the partials are the tangent rules of the interpreted adjoint
// (sde_adjoint.cuh, tan_op), and a zero adjoint propagates nothing where a
// partial may be infinite (no 0 * inf)
std::string op_reverse(uint32_t op) {
    const int code = op & 0xff, d = (op >> 8) & 0xff, ia = (op >> 16) & 0xff, ib = op >> 24;
    if (code == SDE_UOP_CONST) return "";
    const std::string D = "b[" + std::to_string(d) + "]", BA = "b[" + std::to_string(ia) + "]",
                      BB = "b[" + std::to_string(ib) + "]", RA = "r[" + std::to_string(ia) + "]",
                      RB = "r[" + std::to_string(ib) + "]", RD = "r[" + std::to_string(d) + "]";
    auto guarded = [&](const std::string &body) { return "if (" + D + " != R(0)) { " + body + " }"; };
    switch (code) {
    case SDE_UOP_ADD: return BA + " += " + D + "; " + BB + " += " + D + ";";
    case SDE_UOP_SUB: return BA + " += " + D + "; " + BB + " -= " + D + ";";
    case SDE_UOP_MUL: return guarded(BA + " += " + D + " * " + RB + "; " + BB + " += " + D + " * " + RA + ";");
    case SDE_UOP_DIV:
        return guarded("const R q_ = " + D + " / " + RB + "; " + BA + " += q_; " + BB + " -= q_ * " + RD + ";");
    case SDE_UOP_NEG: return BA + " -= " + D + ";";
    case SDE_UOP_ABS: return BA + " += " + RA + " < R(0) ? -" + D + " : " + D + ";";
    case SDE_UOP_EXP: return guarded(BA + " += " + D + " * " + RD + ";");
    case SDE_UOP_LOG: return guarded(BA + " += " + D + " / " + RA + ";");
    case SDE_UOP_SQRT: return "if (" + RD + " > R(0)) " + BA + " += " + D + " * (R(0.5) / " + RD + ");";
    case SDE_UOP_MAX: return "if (" + RA + " >= " + RB + ") " + BA + " += " + D + "; else " + BB + " += " + D + ";";
    case SDE_UOP_MIN: return "if (" + RA + " <= " + RB + ") " + BA + " += " + D + "; else " + BB + " += " + D + ";";
    case SDE_UOP_SIN: return BA + " += " + D + " * F::cos_(" + RA + ");";
    case SDE_UOP_COS: return BA + " -= " + D + " * F::sin_(" + RA + ");";
    case SDE_UOP_TAN: return guarded(BA + " += " + D + " * (R(1) + " + RD + " * " + RD + ");");
    case SDE_UOP_TANH: return BA + " += " + D + " * (R(1) - " + RD + " * " + RD + ");";
    case SDE_UOP_POW:   // d(a^b)/da = b a^(b-1), a^b / a where a > 0 (no second power)
        return guarded("const R pa_ = " + RA + " > R(0) ? " + RD + " / " + RA + " : F::pow_(" + RA + ", " + RB +
                       " - R(1)); " + BA + " += " + D + " * (" + RB + " * pa_); if (" + RA + " > R(0)) " + BB +
                       " += " + D + " * (" + RD + " * F::log_(" + RA + "));");
    case SDE_UOP_EXPM1: return guarded(BA + " += " + D + " * (" + RD + " + R(1));");
    case SDE_UOP_LOG1P: return guarded(BA + " += " + D + " / (R(1) + " + RA + ");");
    case SDE_UOP_ARCTAN: return BA + " += " + D + " / (R(1) + " + RA + " * " + RA + ");";
    default: return BA + " += " + D + ";";   // SDE_UOP_COPY
    }
}

// UserJitAdj<R>: the parameters read and the sources present as
// constants (UserJitFn<R> holds the terms' sources), and back(): at the
// states xs before a step, with the step's increments dz[e][i] of each
// term, adds to the adjoints xb of the states d(x' . xb)/dx - xb, and to pb
// d(x' . xb)/dp, where x'_e = x_e + sum_i A_ei(t, x, p) dz[e][i]: one value
// pass of the program, the terms' adjoints xb_e dz[e][i], then the
// instructions in reverse order
std::string adj_struct(const SdeUserProgram &u, const char *rt) {
    bool has[4] = {false, false, false, false};
    for (int i = 0; i < u.n_terms; ++i) has[u.term_source[i]] = true;
    std::string s = "template <> struct UserJitAdj<";
    s += rt;
    s += "> {\n  typedef ";
    s += rt;
    s += " R;\n  static constexpr int NEQ = " + std::to_string(u.n_eq) + ", NT = " + std::to_string(u.n_terms) +
         ", NP = " + std::to_string(params_read(u)) + ";\n";
    s += std::string("  static constexpr bool HAS_DW = ") + (has[SDE_SRC_DW] ? "true" : "false") +
         ", HAS_DN = " + (has[SDE_SRC_DN] ? "true" : "false") + ", HAS_DJ = " + (has[SDE_SRC_DJ] ? "true" : "false") +
         ";\n";
    s += "  static __device__ __forceinline__ void back(const R (&xs)[NEQ], R t, const R (&p)[6],"
         " const R (&dz)[NEQ][SDE_USER_MAX_TERMS], R (&xb)[NEQ], R (&pb)[6]) {\n"
         "    typedef Ar<R> A;\n    typedef UFn<R> F;\n    R r[SDE_USER_MAX_REGS], b[SDE_USER_MAX_REGS];\n"
         "#pragma unroll\n    for (int i = 0; i < SDE_USER_MAX_REGS; ++i) b[i] = R(0);\n"
         "    r[0] = xs[0];\n    r[1] = t;\n";
    for (int i = 0; i < 6; ++i) s += "    r[" + std::to_string(2 + i) + "] = p[" + std::to_string(i) + "];\n";
    for (int e = 1; e < u.n_eq; ++e) s += "    r[" + std::to_string(7 + e) + "] = xs[" + std::to_string(e) + "];\n";
    for (int i = 0; i < u.n_ops; ++i) s += "    " + op_statement(u, u.ops[i]) + "\n";
    for (int e = 0; e < u.n_eq; ++e)
        for (int i = 0; i < u.n_terms; ++i)
            s += "    b[" + std::to_string(u.term_register[e][i]) + "] += xb[" + std::to_string(e) + "] * dz[" +
                 std::to_string(e) + "][" + std::to_string(i) + "];\n";
    for (int i = u.n_ops - 1; i >= 0; --i) {
        const std::string st = op_reverse(u.ops[i]);
        if (!st.empty()) s += "    " + st + "\n";
    }
    for (int e = 0; e < u.n_eq; ++e)
        s += "    xb[" + std::to_string(e) + "] += b[" + std::to_string(e == 0 ? 0 : 7 + e) + "];\n";
    for (int j = 0; j < 6; ++j) s += "    pb[" + std::to_string(j) + "] += b[" + std::to_string(2 + j) + "];\n";
    s += "  }\n};\n";
    return s;
}

// resident blocks the adjoint kernel is compiled for: FP32 groups of up to
// two states at three 256-thread blocks per SM
int adj_user_min_blocks(bool fp64, int mg) {
    if (mg <= 2) return fp64 ? 2 : 3;
    return mg <= 4 ? 2 : 1;
}

std::string adj_kernel_name(const char *rt, int maxm, int mg, int minb) {
    char buf[160];
    snprintf(buf, sizeof buf, "sdegpu::sde_adj_user_kernel<%s, %d, %d, %d>", rt, maxm, mg, minb);
    return buf;
}

// the adjoint kernel of a program for groups of mg states (sde_adj_user.cuh)
std::string jit_adj_source(const SdeUserProgram &u, const char *rt, int maxm, int mg, int minb) {
    return "#include \"sde_adj_user.cuh\"\nnamespace sdegpu {\n" + coefs_struct(u, rt) + adj_struct(u, rt) +
           "template __global__ void " + adj_kernel_name(rt, maxm, mg, minb) + "(const __grid_constant__ AdjArgs<" +
           rt + ">);\n}  // namespace sdegpu\n";
}

struct Entry {
    cudaLibrary_t lib;
    cudaKernel_t kernel;
    int bps;
};

std::mutex g_cache_mu;
std::map<std::string, Entry> g_cache;

// compile src to a cubin; the kernel's lowered name in *low
int compile_cubin(const std::string &src, const std::string &name, std::vector<char> *cubin, std::string *low,
                  std::string *err) {
    Nvrtc &N = nvrtc();
    if (!N.ok) {
        *err = "NVRTC is not available for compiling user SDE programs";
        return SDE_ERR_UNSUPPORTED;
    }
    if (const char *dir = getenv("SDEPY_GB300_JIT_DUMP")) {
        char path[4096];
        snprintf(path, sizeof path, "%s/sde_jit_%016zx.cu", dir, std::hash<std::string>()(src));
        if (FILE *f = fopen(path, "w")) {
            fprintf(f, "// %s\n%s", name.c_str(), src.c_str());
            fclose(f);
        }
    }
    nvrtcProgram prog;
    if (N.create(&prog, src.c_str(), "sde_user_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        *err = "nvrtcCreateProgram failed";
        return SDE_ERR_CUDA;
    }
    N.add_name(prog, name.c_str());
    const std::string inc = "-I" + N.include_dir;
    // the library build's target and language (sm_103a, C++17; no fast math)
    const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device", inc.c_str()};
    const nvrtcResult rc = N.compile(prog, 4, opts);
    if (rc != NVRTC_SUCCESS) {
        size_t n = 0;
        N.log_size(prog, &n);
        std::vector<char> log(n + 1, 0);
        N.log(prog, log.data());
        *err = "compiling the user SDE program: " + std::string(log.data()).substr(0, 600);
        N.destroy(&prog);
        return SDE_ERR_UNSUPPORTED;
    }
    const char *lowered = nullptr;
    size_t nb = 0;
    N.lowered(prog, name.c_str(), &lowered);
    N.cubin_size(prog, &nb);
    cubin->assign(nb, 0);
    N.cubin(prog, cubin->data());
    *low = lowered ? lowered : "";
    N.destroy(&prog);
    return SDE_OK;
}

}  // namespace

bool jit_available() { return nvrtc().ok; }

int jit_compile_check(const SdeUserProgram &u, bool fp64, int maxm, bool inject, bool jumps, std::string *err) {
    const char *rt = fp64 ? "double" : "float";
    const int model = u.n_eq > 1 ? SDE_MODEL_USER_SYS_JIT : SDE_MODEL_USER_JIT;
    std::vector<char> cubin;
    std::string low;
    return compile_cubin(jit_source(u, rt, model, maxm, inject, jumps), kernel_name(rt, model, maxm, inject, jumps),
                         &cubin, &low, err);
}

// the kernel `name` of `src`, compiled and loaded once per process
static int cached_kernel(const std::string &src, const std::string &name, cudaKernel_t *kernel, int *bps,
                         std::string *err) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_cache.find(src);
    if (it != g_cache.end()) {
        *kernel = it->second.kernel;
        *bps = it->second.bps;
        return SDE_OK;
    }
    std::vector<char> cubin;
    std::string low;
    int rc;
    if ((rc = compile_cubin(src, name, &cubin, &low, err))) return rc;
    Entry e;
    if (cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
        cudaLibraryGetKernel(&e.kernel, e.lib, low.c_str()) != cudaSuccess) {
        *err = std::string("loading the compiled user SDE program: ") + cudaGetErrorString(cudaGetLastError());
        return SDE_ERR_CUDA;
    }
    e.bps = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e.bps, (const void *)e.kernel, BLOCK, 0) != cudaSuccess ||
        e.bps < 1) {
        cudaGetLastError();
        e.bps = 1;
    }
    g_cache.emplace(src, e);
    *kernel = e.kernel;
    *bps = e.bps;
    return SDE_OK;
}

static int maxm_of_group(int mg) { return mg <= 1 ? 1 : mg <= 2 ? 2 : mg <= 4 ? 4 : 8; }

int jit_compile_check_adjoint(const SdeUserProgram &u, bool fp64, int mg, std::string *err) {
    const char *rt = fp64 ? "double" : "float";
    const int maxm = maxm_of_group(mg), minb = adj_user_min_blocks(fp64, mg);
    std::vector<char> cubin;
    std::string low;
    return compile_cubin(jit_adj_source(u, rt, maxm, mg, minb), adj_kernel_name(rt, maxm, mg, minb), &cubin, &low,
                         err);
}

int jit_fwd_kernel(const SdeUserProgram &u, bool fp64, int maxm, bool inject, bool jumps, cudaKernel_t *kernel,
                   int *bps, std::string *err) {
    const char *rt = fp64 ? "double" : "float";
    const int model = u.n_eq > 1 ? SDE_MODEL_USER_SYS_JIT : SDE_MODEL_USER_JIT;
    return cached_kernel(jit_source(u, rt, model, maxm, inject, jumps), kernel_name(rt, model, maxm, inject, jumps),
                         kernel, bps, err);
}

int jit_adj_kernel(const SdeUserProgram &u, bool fp64, int mg, cudaKernel_t *kernel, std::string *err) {
    const char *rt = fp64 ? "double" : "float";
    const int maxm = maxm_of_group(mg), minb = adj_user_min_blocks(fp64, mg);
    int bps;
    return cached_kernel(jit_adj_source(u, rt, maxm, mg, minb), adj_kernel_name(rt, maxm, mg, minb), kernel, &bps,
                         err);
}

}  // namespace sdegpu

extern "C" int32_t sde_jit_available(void) { return sdegpu::jit_available() ? 1 : 0; }

extern "C" int32_t sde_jit_compile_adjoint(const SdeUserProgram *program, int32_t precision, int32_t group_size,
                                           char *log, int32_t len) {
    std::string err;
    int rc = SDE_ERR_INVALID;
    if (!program || group_size < 1 || group_size > 8 || program->n_eq < 1 || program->n_eq > SDE_USER_MAX_EQ ||
        group_size % program->n_eq || program->n_ops < 0 || program->n_ops > SDE_USER_MAX_OPS ||
        program->n_terms < 0 || program->n_terms > SDE_USER_MAX_TERMS) {
        err = "invalid program or group size (1..8, whole components of a system)";
    } else {
        rc = sdegpu::jit_compile_check_adjoint(*program, precision == SDE_FP64, group_size, &err);
    }
    if (log && len > 0) {
        strncpy(log, err.c_str(), (size_t)len - 1);
        log[len - 1] = 0;
    }
    return rc;
}

extern "C" int32_t sde_jit_compile(const SdeUserProgram *program, int32_t precision, int32_t group_size,
                                   int32_t injected, int32_t jumps, char *log, int32_t len) {
    std::string err;
    int rc = SDE_ERR_INVALID;
    if (!program || group_size < 1 || group_size > SDE_MAX_GROUP || program->n_eq < 1 ||
        program->n_eq > SDE_USER_MAX_EQ || program->n_ops < 0 || program->n_ops > SDE_USER_MAX_OPS ||
        program->n_terms < 0 || program->n_terms > SDE_USER_MAX_TERMS) {
        err = "invalid program or group size";
    } else {
        const int maxm = group_size <= 1 ? 1 : group_size <= 2 ? 2 : group_size <= 4 ? 4 : group_size <= 8 ? 8 : 16;
        rc = sdegpu::jit_compile_check(*program, precision == SDE_FP64, maxm, injected != 0, jumps != 0, &err);
    }
    if (log && len > 0) {
        strncpy(log, err.c_str(), (size_t)len - 1);
        log[len - 1] = 0;
    }
    return rc;
}
