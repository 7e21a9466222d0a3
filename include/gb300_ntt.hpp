// gb300_ntt.hpp -- C++ host classes over the C ABI, mirroring the reference's
// ADF graph classes (same template parameters, same compile-time checks,
// same init/run/end lifecycle).  Header-only; link with libgb300ntt.so.
//
//   reference (AIE1)                                   here
//   NTT<LENGTH,MODULUS,ROOT,ROW,COL,NTT_TYPE>          gb300ntt::NTT<LENGTH,MODULUS,ROOT,NTT_TYPE>
//     src/ntt.h:43
//   NTT_INT32<LENGTH,MODULUS,ROOT,ROW,COL,TYPE>        gb300ntt::NTT_INT32<LENGTH,MODULUS,ROOT,TYPE>
//     src/ntt_int32.h:27
//   NTT_R4<LENGTH,MODULUS,ROOT,ROW,COL,TYPE>           gb300ntt::NTT_R4<LENGTH,MODULUS,ROOT,TYPE>
//     src/ntt_r4.h:30
//   NTT_R8<LENGTH,MODULUS,ROOT>                        gb300ntt::NTT_R8<LENGTH,MODULUS,ROOT,STAGES>
//     src/ntt_r8.h:22
//   BITREVERSE<LENGTH>                                 gb300ntt::BITREVERSE<LENGTH>
//     src/standalone_units.h:17
//   FULL_BARRETT_MULTIPLICATION<LENGTH,MODULUS,FACTOR> gb300ntt::FULL_BARRETT_MULTIPLICATION<...>
//     src/standalone_units.h:40
//
// The tile placement parameters (STARTROW, STARTCOL) have no GPU meaning and
// are dropped.  The ports in_data / out_data are device pointers; run(N)
// transforms N polynomials (one per graph iteration in the reference).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>

#include "gb300_ntt.h"

namespace gb300ntt {

// ---- compile-time number theory (src/auxiliary.h) ----

constexpr uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (unsigned __int128)a * b % m; }

// smallest L with ROOT^(2^L) == 1 mod MODULUS, or -1 (DETERMINE_LOG_ROOT_SIZE, auxiliary.h:35-46)
constexpr int log_root_size(uint64_t modulus, uint64_t root) {
    uint64_t x = root % modulus;
    for (int L = 0; L <= 100; ++L) {
        if (x == 1) return L;
        x = mulmod(x, x, modulus);
    }
    return -1;
}

constexpr int log2_exact(uint64_t n) {
    int l = 0;
    while ((uint64_t(1) << l) < n) ++l;
    return (uint64_t(1) << l) == n ? l : -1;
}

// n^-1 mod m (ExtendedGCD, auxiliary.h:66-79)
constexpr int64_t mod_inverse(int64_t n, int64_t m) {
    int64_t a = n, b = m, x0 = 1, x1 = 0;
    while (b) {
        int64_t q = a / b, t = a % b;
        a = b; b = t;
        t = x1; x1 = x0 - q * x1; x0 = t;
    }
    return (x0 % m + m) % m;
}

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
    int code;
};

inline void check(int rc) {
    if (rc != GBNTT_OK)
        throw Error(rc, std::string(gbntt_status_string(rc)) + ": " + gbntt_last_error());
}

// ---- graph base: plan lifecycle and ports ----

class graph {
public:
    graph(int kind, uint32_t n, int64_t q, int64_t root, int64_t factor, uint32_t flags)
        : kind_(kind), n_(n), q_(q), root_(root), factor_(factor), flags_(flags) {}
    graph(const graph&) = delete;
    graph& operator=(const graph&) = delete;
    virtual ~graph() { end(); }

    // graph.init(): build the tables and upload them (src/project.cpp:162)
    void init() {
        if (!plan_) check(gbntt_plan_create(&plan_, kind_, n_, q_, root_, factor_, flags_));
    }
    // graph.run(N): N polynomials from in_data to out_data (src/project.cpp:163)
    void run(uint64_t iterations, void* stream = nullptr) {
        init();
        check(gbntt_execute(plan_, in_data, out_data, iterations, stream));
    }
    // graph.end(): release the tables (src/project.cpp:164)
    void end() {
        if (plan_) {
            gbntt_plan_destroy(plan_);
            plan_ = nullptr;
        }
    }
    gbntt_plan* plan() { return plan_; }

    const void* in_data = nullptr;   // input port: device pointer
    void* out_data = nullptr;        // output port: device pointer

protected:
    int kind_;
    uint32_t n_;
    int64_t q_, root_, factor_;
    uint32_t flags_;
    gbntt_plan* plan_ = nullptr;
};

enum class NTT_TYPE { TYPE_NTT_NO_to_BO, TYPE_INTT_BO_to_NO };                 // src/ntt.h:30-33
enum class NTT_INT32_TYPE { FORWARD_CT_NO_TO_BO, INVERSE_GS_BO_TO_NO };        // src/ntt_int32.h:19-22
enum class NTT_R4_TYPE { FORWARD_CT_NO_TO_BO, INVERSE_BO_TO_NO };             // src/ntt_r4.h:23-25 (+ inverse)

template <uint32_t LENGTH, uint32_t MODULUS, uint32_t ROOT>
struct ntt_params {
    static_assert(log2_exact(LENGTH) > 0, "LENGTH must be a power of two");
    static constexpr int NTT_MODULUS_ = MODULUS;
    static constexpr int NTT_ROOT_ = ROOT;
    static constexpr int NTT_LENGTH = LENGTH;
    static constexpr int LENGTH_MOD_INV = (int)mod_inverse(LENGTH, MODULUS);
    static constexpr int MAX_NO_OF_LAYERS = log_root_size(MODULUS, ROOT);
    static_assert(MAX_NO_OF_LAYERS >= 0, "ROOT is not correct");
    static_assert(MAX_NO_OF_LAYERS == log2_exact(LENGTH), "ROOT must have order LENGTH");
    static constexpr int LAYERS = MAX_NO_OF_LAYERS;
};

// Radix-2 int16 pipeline (src/ntt.h:43).
template <uint32_t LENGTH, uint32_t MODULUS, uint32_t ROOT, NTT_TYPE TYPE = NTT_TYPE::TYPE_NTT_NO_to_BO>
class NTT : public graph, public ntt_params<LENGTH, MODULUS, ROOT> {
    static_assert(3 * (uint64_t)MODULUS < 65536, "MODULUS must be below 2^16 / 3 (lazy reduction bound)");
public:
    static constexpr bool INVERSE_TRANSFORM = TYPE == NTT_TYPE::TYPE_INTT_BO_to_NO;
    static constexpr int K_BARRETT = 16;
    typedef int16_t DATA_TYPE;
    explicit NTT(uint32_t flags = 0)
        : graph(INVERSE_TRANSFORM ? GBNTT_R2_I16_INV : GBNTT_R2_I16_FWD, LENGTH, MODULUS, ROOT, 0, flags) {}
};

// Radix-2 int32 pipeline (src/ntt_int32.h:27).
template <uint32_t LENGTH, uint32_t MODULUS, uint32_t ROOT,
          NTT_INT32_TYPE TYPE = NTT_INT32_TYPE::FORWARD_CT_NO_TO_BO>
class NTT_INT32 : public graph, public ntt_params<LENGTH, MODULUS, ROOT> {
    static_assert(3 * (uint64_t)MODULUS < (uint64_t(1) << 32), "MODULUS must be below 2^32 / 3");
public:
    static constexpr bool INVERSE_TRANSFORM = TYPE == NTT_INT32_TYPE::INVERSE_GS_BO_TO_NO;
    static constexpr unsigned K_BARRETT = 32;
    typedef int32_t DATA_TYPE;
    explicit NTT_INT32(uint32_t flags = 0)
        : graph(INVERSE_TRANSFORM ? GBNTT_R2_I32_INV : GBNTT_R2_I32_FWD, LENGTH, MODULUS, ROOT, 0, flags) {}
};

// Radix-4 int16 pipeline (src/ntt_r4.h:30).
template <uint32_t LENGTH, uint32_t MODULUS, uint32_t ROOT, NTT_R4_TYPE TYPE = NTT_R4_TYPE::FORWARD_CT_NO_TO_BO>
class NTT_R4 : public graph, public ntt_params<LENGTH, MODULUS, ROOT> {
    static_assert(log2_exact(LENGTH) % 2 == 0, "MUST BE EVEN AMOUNT OF LAYERS");   // src/ntt_r4.h:62-63
public:
    static constexpr int NO_OF_R4_LAYERS = log2_exact(LENGTH) / 2;
    typedef int16_t DATA_TYPE;
    explicit NTT_R4(uint32_t flags = 0)
        : graph(TYPE == NTT_R4_TYPE::FORWARD_CT_NO_TO_BO ? GBNTT_R4_I16_FWD : GBNTT_R4_I16_INV, LENGTH, MODULUS,
                ROOT, 0, flags) {}
};

// Radix-8 int16 (src/ntt_r8.h:22).  STAGES = 1: the reference graph, one
// stage with its float-derived multipliers; STAGES = 0: every stage chained.
template <uint32_t LENGTH, uint32_t MODULUS, uint32_t ROOT, int STAGES = 1>
class NTT_R8 : public graph, public ntt_params<LENGTH, MODULUS, ROOT> {
public:
    typedef int16_t DATA_TYPE;
    explicit NTT_R8(uint32_t flags = 0)
        : graph(STAGES == 1 ? GBNTT_R8_I16_STAGE : GBNTT_R8_I16_FWD, LENGTH, MODULUS, ROOT, 0, flags) {}
};

// Bit-reversal unit (src/standalone_units.h:17, bitreverse_kernels.cc:58).
template <uint32_t LENGTH>
class BITREVERSE : public graph {
    static_assert(LENGTH == 256 || LENGTH == 512 || LENGTH == 1024 || LENGTH == 2048 || LENGTH == 4096,
                  "LENGTH must be 256,512,1024,2048 or 4096");
public:
    BITREVERSE() : graph(GBNTT_BITREV_I16, LENGTH, 0, 0, 0, 0) {}
};

// Full Barrett multiplication by FACTOR (src/standalone_units.h:40).
template <uint32_t LENGTH, uint32_t MODULUS, uint32_t FACTOR>
class FULL_BARRETT_MULTIPLICATION : public graph {
    static_assert(FACTOR < MODULUS, "FACTOR must be reduced");
public:
    FULL_BARRETT_MULTIPLICATION() : graph(GBNTT_FULL_BARRETT_I16, LENGTH, MODULUS, 0, FACTOR, 0) {}
};

// Parameters of the reference (src/project.cpp:47-51).
constexpr uint32_t Q_INT16 = 12289, ROOT_INT16 = 41;
constexpr uint32_t Q_INT32 = 1073707009, ROOT_INT32 = 992735929;

}  // namespace gb300ntt
