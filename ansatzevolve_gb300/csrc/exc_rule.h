// Excitation rule shared by host setup code and device kernels.
//
// One excitation is four signed spin-orbital indices (0-based, -1 = absent):
// a single "a b -1 -1" is a^+_a a_b, a double "a b c d" is a^+_a a^+_b a_c a_d.
// Applied to a determinant bitstring it either does nothing, pairs the determinant
// with a partner and a +/-1 sign, or (number / density-density operators, complex
// mode only) multiplies it by a phase.  The rule restates fusedevolve.cpp:27-145 of
// the reference (identical to stateRotate::getLieAlgebraMatrix, operatorpool.cpp:40-127):
//   signMask = XOR of ((1<<x)-1) over the operator's indices, those bits cleared;
//   phase    = (-1)^popc(state & signMask) * (-1)^[a>b] * (-1)^[c>d];
//   state holds every annihilated orbital and none of the created ones (after the
//   annihilation) -> partner = state ^ ann ^ cre, sign = +phase;
//   state holds every created orbital and none of the annihilated ones
//                -> partner = state ^ cre ^ ann, sign = -phase.
// The generator G of the rotation exp(theta G) then acts as (G v)_z = sign(z) v_partner(z),
// which is antisymmetric (sign(partner) = -sign(z)) because the two determinants agree
// outside the operator's orbitals.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define AE_HD __host__ __device__ __forceinline__
#else
#define AE_HD inline
#endif

namespace ae {

struct ExcCode {
    uint32_t create;     // created orbitals
    uint32_t annihilate; // annihilated orbitals
    uint32_t signmask;   // orbitals strictly between the operator's indices (parity mask)
    int32_t perm;        // +1 / -1 ordering phase of the double
    int32_t diagonal;    // 1: number / density-density operator (create == annihilate)
    int32_t valid;       // 0: identity operator (a < 0 && b < 0)
};

AE_HD int ae_popc(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

AE_HD ExcCode make_exc_code(int a, int b, int c, int d)
{
    ExcCode e{0u, 0u, 0u, 1, 0, 1};
    if (a < 0 && b < 0) { e.valid = 0; return e; }
    if (c > -1 && d > -1) {
        e.create = (1u << a) | (1u << b);
        e.annihilate = (1u << c) | (1u << d);
        uint32_t m = ((1u << a) - 1u) ^ ((1u << b) - 1u) ^ ((1u << c) - 1u) ^ ((1u << d) - 1u);
        e.signmask = m & ~(e.create | e.annihilate);
        e.perm = ((a > b) ? -1 : 1) * ((c > d) ? -1 : 1);
    } else {
        e.create = 1u << a;
        e.annihilate = 1u << b;
        uint32_t m = ((1u << a) - 1u) ^ ((1u << b) - 1u);
        e.signmask = m & ~(e.create | e.annihilate);
        e.perm = 1;
    }
    e.diagonal = e.create == e.annihilate;
    return e;
}

// 0 inactive, 1 paired (partner, sign), 2 diagonal phase (sign = +1).
AE_HD int apply_exc(const ExcCode &e, uint32_t state, uint32_t &partner, int &sign)
{
    partner = state;
    sign = 1;
    if (!e.valid) return 0;
    uint32_t m = state & (e.create | e.annihilate);
    if (e.diagonal) return (m & e.annihilate) == e.annihilate ? 2 : 0;
    int ph = e.perm * ((ae_popc(state & e.signmask) & 1) ? -1 : 1);
    if ((m & e.annihilate) == e.annihilate && ((m ^ e.annihilate) & e.create) == 0) {
        partner = state ^ e.annihilate ^ e.create;
        sign = ph;
        return 1;
    }
    if ((m & e.create) == e.create && ((m ^ e.create) & e.annihilate) == 0) {
        partner = state ^ e.create ^ e.annihilate;
        sign = -ph;
        return 1;
    }
    return 0;
}

// Sign only, for a determinant already known to be active for a paired excitation.
AE_HD int exc_sign(const ExcCode &e, uint32_t state)
{
    int ph = e.perm * ((ae_popc(state & e.signmask) & 1) ? -1 : 1);
    return ((state & e.annihilate) == e.annihilate && !((state ^ e.annihilate) & e.create)) ? ph : -ph;
}

// Hamiltonian term a^+ a^+ a a / a^+ a with its parity mask (hamiltonianmatrix.h:11-20).
struct HamOp {
    uint32_t create, destroy, signmask;
};

}  // namespace ae
