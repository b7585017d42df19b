// elem_io.cuh - how an elementwise kernel thread reads and writes one
// element: the caller's dense little-endian byte strings (the ABI's layout,
// reference host/include/cft.h:1172-1174) as 16-byte vectors (fp256: two,
// fp128: one), an 8-byte pair (fp64) or one word (fp32).
#pragma once
#include "cftg_internal.h"
#include "simple_ops.cuh"

namespace cftg {

template <int W>
SFD void load_elem(const uint32_t *__restrict__ base, size_t j, uint32_t (&x)[W])
{
    const uint32_t *p = base + j * W;
    if constexpr (W == 8) {
        const uint4 v0 = reinterpret_cast<const uint4 *>(p)[0];
        const uint4 v1 = reinterpret_cast<const uint4 *>(p)[1];
        x[0] = v0.x; x[1] = v0.y; x[2] = v0.z; x[3] = v0.w;
        x[4] = v1.x; x[5] = v1.y; x[6] = v1.z; x[7] = v1.w;
    } else if constexpr (W == 4) {
        const uint4 v = reinterpret_cast<const uint4 *>(p)[0];
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
    } else if constexpr (W == 2) {
        const uint2 v = reinterpret_cast<const uint2 *>(p)[0];
        x[0] = v.x; x[1] = v.y;
    } else {
        x[0] = p[0];
    }
}

template <int W>
SFD void store_elem(uint32_t *__restrict__ base, size_t j, const uint32_t (&x)[W])
{
    uint32_t *p = base + j * W;
    if constexpr (W == 8) {
        reinterpret_cast<uint4 *>(p)[0] = make_uint4(x[0], x[1], x[2], x[3]);
        reinterpret_cast<uint4 *>(p)[1] = make_uint4(x[4], x[5], x[6], x[7]);
    } else if constexpr (W == 4) {
        reinterpret_cast<uint4 *>(p)[0] = make_uint4(x[0], x[1], x[2], x[3]);
    } else if constexpr (W == 2) {
        reinterpret_cast<uint2 *>(p)[0] = make_uint2(x[0], x[1]);
    } else {
        p[0] = x[0];
    }
}

// Operand r of element i: +0 for a NULL operand or a CFT_IDX_NONE index,
// element 0 for a scalar, source[idx[i]] through a table, else element i.
template <int W>
SFD void fetch(const void *src, bool scalar, const uint32_t *idx, size_t i, uint32_t (&x)[W])
{
    if (!src) {
        sfw::zero(x);
        return;
    }
    size_t j = scalar ? 0 : i;
    if (idx) {
        const uint32_t t = idx[i];
        if (t == 0xFFFFFFFFu) {
            sfw::zero(x);
            return;
        }
        j = t;
    }
    load_elem<W>(static_cast<const uint32_t *>(src), j, x);
}


// One element of a (format, kind) launch: o and fl from a, b, c (operands
// the kind does not read are +0).
template <int FMT, int KIND, int W>
SFD void compute_elem(int op, int rnd, uint32_t (&a)[W], uint32_t (&b)[W], uint32_t (&c)[W],
                      uint32_t (&o)[W], uint32_t &fl)
{
    if constexpr (KIND <= K_MUL) sf::arith<FMT, KIND>(a, b, c, rnd, o, fl);
    else if constexpr (KIND == K_DIV) sf::div<FMT>(a, b, rnd, o, fl);
    else if constexpr (KIND == K_SQRT) sf::sqrt<FMT>(a, rnd, o, fl);
    else sf::simple<FMT>(op, a, b, c, o, fl);
}

}  // namespace cftg
