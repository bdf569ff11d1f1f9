/*
 * ref_probe.cpp — runs the REFERENCE's own host-callable code on the CPU to
 * pin the oracle.  TEST INFRASTRUCTURE ONLY (built into oracle/_ref/, which is
 * not committed; its output is committed as tests/golden/ fixtures).
 *
 * It includes the reference headers where they lie (-I <reference>/include)
 * and calls, on the host:
 *   rsort::detail::radix_traits<T, IsLD>::twiddle_in / twiddle_out
 *       (include/rsort/detail/tuning.cuh:352-384)
 *   rsort::detail::mix32 (include/rsort/detail/utils.cuh:228-242)
 *   rsort::detail::set_seed_radix (include/rsort/detail/utils.cuh:435-437)
 *
 * Input: lines "<type> <hex bits>" on stdin, type one of u8 u16 u32 u64 u128
 * i8 i16 i32 i64 i128 f32 f64 f128, bits as big-endian hex of the key's raw
 * bytes (little-endian in memory).  Output per line:
 *   "<type> <bits> <in_asc> <in_desc> <out_asc(bits)> <out_desc(bits)>"
 * all hex.  A line "mix32 <hex>" prints "mix32 <hex> <mix32(hex)>", a line
 * "seed <i>" prints "seed <i> <set_seed_radix(i)>".
 *
 * The reference's headers use a handful of CUDA device builtins in functions
 * this probe never calls; host stand-ins below only let them parse.  The
 * four bit-cast intrinsics ARE used by the float twiddle and are defined here
 * as memcpy bit casts, which is what they are.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>

#include <cuda_runtime.h>

unsigned int __float_as_uint(float x) { unsigned int u; std::memcpy(&u, &x, 4); return u; }
float __uint_as_float(unsigned int x) { float f; std::memcpy(&f, &x, 4); return f; }
long long __double_as_longlong(double x) { long long u; std::memcpy(&u, &x, 8); return u; }
double __longlong_as_double(long long x) { double f; std::memcpy(&f, &x, 8); return f; }

// Parse-only stand-ins for device builtins referenced by unused helpers.
struct ProbeDim3 { unsigned x, y, z; };
static ProbeDim3 threadIdx, blockIdx, blockDim;
template <class T> T atomicAdd(T* p, T v) { T o = *p; *p += v; return o; }
inline int atomicExch(int* p, int v) { int o = *p; *p = v; return o; }

#include "rsort/detail/utils.cuh"

using rsort::detail::radix_traits;
using u128 = unsigned __int128;

static u128 parse_hex(const std::string& s) {
    u128 v = 0;
    for (char c : s) {
        int d = (c >= '0' && c <= '9') ? c - '0' : (c >= 'a' && c <= 'f') ? c - 'a' + 10 : c - 'A' + 10;
        v = (v << 4) | u128(d);
    }
    return v;
}

static std::string hex(u128 v, int bytes) {
    std::string s(bytes * 2, '0');
    for (int i = bytes * 2 - 1; i >= 0; --i) {
        s[i] = "0123456789abcdef"[unsigned(v & 15)];
        v >>= 4;
    }
    return s;
}

template <class T, bool IsLD = false>
static void run(const char* name, u128 raw) {
    using Tr = radix_traits<T, IsLD>;
    using U = typename Tr::unsigned_of;
    constexpr int B = sizeof(T);
    T x;
    U rawu = U(raw);
    std::memcpy(&x, &rawu, B);
    U ia = Tr::template twiddle_in<false>(x);
    U id = Tr::template twiddle_in<true>(x);
    T oa = Tr::template twiddle_out<false>(rawu);
    T od = Tr::template twiddle_out<true>(rawu);
    U oau, odu;
    std::memcpy(&oau, &oa, B);
    std::memcpy(&odu, &od, B);
    std::printf("%s %s %s %s %s %s\n", name, hex(rawu, B).c_str(), hex(ia, B).c_str(),
                hex(id, B).c_str(), hex(oau, B).c_str(), hex(odu, B).c_str());
}

int main() {
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream is(line);
        std::string t, v;
        if (!(is >> t >> v)) continue;
        if (t == "mix32") {
            uint32_t x = uint32_t(parse_hex(v));
            std::printf("mix32 %08x %08x\n", x, rsort::detail::mix32(x));
            continue;
        }
        if (t == "seed") {
            int i = std::stoi(v);
            std::printf("seed %d %d\n", i, rsort::detail::set_seed_radix(i));
            continue;
        }
        u128 raw = parse_hex(v);
        if (t == "u8") run<uint8_t>("u8", raw);
        else if (t == "u16") run<uint16_t>("u16", raw);
        else if (t == "u32") run<uint32_t>("u32", raw);
        else if (t == "u64") run<uint64_t>("u64", raw);
        else if (t == "u128") run<u128>("u128", raw);
        else if (t == "i8") run<int8_t>("i8", raw);
        else if (t == "i16") run<int16_t>("i16", raw);
        else if (t == "i32") run<int32_t>("i32", raw);
        else if (t == "i64") run<int64_t>("i64", raw);
        else if (t == "i128") run<__int128>("i128", raw);
        else if (t == "f32") run<float>("f32", raw);
        else if (t == "f64") run<double>("f64", raw);
        // long double: the reference sorts it as unsigned __int128 with the
        // float twiddle (radix_kernel.cuh:351-356, Is_Long_Double = true).
        else if (t == "f128") run<u128, true>("f128", raw);
    }
    return 0;
}
