// midint_compat.hpp -- drop-in C++ replacements for the reference's kernel
// drivers, with the same names, template parameters and argument meaning as
// cuda/main.cu, implemented over the C ABI of midint.h.
//
//   gpuAdd<Base, m>(num_instances, h_as, h_bs, h_rs)       cuda/main.cu:39-44
//   gpuMultiply<Base, m>(num_instances, h_as, h_bs, h_rs)  cuda/main.cu:221-226
//   gpuMulFFT<FftPrime32, M>(num_instances, h_as, h_bs, h_rs) cuda/main.cu:415-420
//
// Base is U64bits or U32bits (the limb traits of cuda/ker-helpers.cu.h:12-28),
// m the size in Base::uint_t limbs, buffers are host memory owned by the
// caller, results are truncated to m limbs exactly as the reference does.
// The differences a caller sees: every function returns the mi_status of the
// call instead of printing CUDA errors and continuing (cuda/helper.h:13-19);
// nothing is printed or timed; gpuMulFFT returns the exact low half of the
// product, which the reference's kernel does not (its validation is disabled,
// cuda/main.cu:729-739).
#ifndef MIDINT_COMPAT_HPP
#define MIDINT_COMPAT_HPP

#include <cstdint>

#include "midint.h"

namespace midint_compat {

struct U64bits {
    using uint_t = uint64_t;
    using sint_t = int64_t;
    using carry_t = uint32_t;
    static const int32_t bits = 64;
    static const uint_t HIGHEST = 0xFFFFFFFFFFFFFFFFull;
};

struct U32bits {
    using uint_t = uint32_t;
    using sint_t = int32_t;
    using carry_t = uint32_t;
    static const int32_t bits = 32;
    static const uint_t HIGHEST = 0xFFFFFFFFu;
};

// The reference's 32-bit NTT prime traits (cuda/ker-fft-mul.cu.h:59-72); only
// its digit types matter here.
struct FftPrime32 {
    using uint_t = uint32_t;
    using uhlf_t = unsigned short;
    static const int32_t bits = 32;
};

namespace detail {
inline mi_status add(U64bits, int n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r) {
    return mi_compat_gpuAdd_u64(n, m, a, b, r);
}
inline mi_status add(U32bits, int n, uint32_t m, const uint32_t* a, const uint32_t* b, uint32_t* r) {
    return mi_compat_gpuAdd_u32(n, m, a, b, r);
}
inline mi_status mul(U64bits, int n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r) {
    return mi_compat_gpuMultiply_u64(n, m, a, b, r);
}
inline mi_status mul(U32bits, int n, uint32_t m, const uint32_t* a, const uint32_t* b, uint32_t* r) {
    return mi_compat_gpuMultiply_u32(n, m, a, b, r);
}
}  // namespace detail

template <class Base, uint32_t m>
mi_status gpuAdd(int num_instances, typename Base::uint_t* h_as, typename Base::uint_t* h_bs,
                 typename Base::uint_t* h_rs) {
    return detail::add(Base{}, num_instances, m, h_as, h_bs, h_rs);
}

template <class Base, int m>
mi_status gpuMultiply(int num_instances, typename Base::uint_t* h_as, typename Base::uint_t* h_bs,
                      typename Base::uint_t* h_rs) {
    return detail::mul(Base{}, num_instances, uint32_t(m), h_as, h_bs, h_rs);
}

template <typename P, uint32_t m>
mi_status gpuMulFFT(int num_instances, typename P::uhlf_t* h_as, typename P::uhlf_t* h_bs,
                    typename P::uint_t* h_rs) {
    static_assert(sizeof(typename P::uhlf_t) == 2, "the FftPrime32 (16-bit digit) shape is provided");
    return mi_compat_gpuMulFFT_u16(num_instances, m, reinterpret_cast<const uint16_t*>(h_as),
                                   reinterpret_cast<const uint16_t*>(h_bs), reinterpret_cast<uint32_t*>(h_rs));
}

}  // namespace midint_compat

#endif  // MIDINT_COMPAT_HPP
