// Variable-time inversion in Fp for public values: Kaliski's almost
// Montgomery inverse (B. S. Kaliski, "The Montgomery inverse and its
// applications", IEEE Trans. Computers 44(8), 1995), phase 1, taking every
// run of trailing zeros in one step, followed by a correction by a table
// constant.  One inversion is ~270 subtract-and-shift iterations on 12-limb
// integers (at most ~390 for 381-bit inputs), against ~570 dependent
// multiplications for Fermat's a^(p-2): a thread finishes it in tens of
// microseconds instead of ~0.45 ms, which is what lets the batch-affine
// bucket rounds invert once per block and round without stalling the GPU.
//
// Phase 1 on U (the Montgomery representation aR, as an integer in [1, p)):
//   u = p, v = U, r = 0, s = 1, k = 0; invariant p = u s + v r (so r, s <= p)
//   strip v's trailing zeros (r = 0 stays 0)
//   loop with u, v odd:
//     u > v:  u = (u - v) >> t, r = r + s, s = s << t, k += t
//     u < v:  v = (v - u) >> t, s = r + s, r = r << t, k += t
//     u = v (= 1):  s = r + s, r = 2 r, k += 1, stop
//   r >= p ? r - p : r,  X = p - r = U^-1 2^k mod p,  381 <= k <= 762.
// Correction: a^-1 in Montgomery form is U^-1 R^2 = X R^2 2^-k; with
// k = 32 a + b that is mont(mont(X, R^3 2^(-32a)), R 2^-b) (two Montgomery
// multiplications by KINV_T1[a] and KINV_T2[b]).
#pragma once
#include "field.cuh"

namespace catmsm {

// KINV_T1[a] = R^3 2^(-32 a) mod p, KINV_T2[b] = R 2^(-b) mod p (little-endian
// 32-bit words; R = 2^384).  Checked against a big-integer recomputation by
// tests/test_capi_symbols.py.
__device__ __constant__ static const uint32_t KINV_T1[25][12] = {
    {0xd94ca1e0u, 0xed48ac6bu, 0x03a7adf8u, 0x315f831eu, 0x615e29ddu, 0x9a53352au, 0x921e1761u, 0x34c04e5eu, 0x65724728u, 0x2512d435u, 0x91755d4du, 0x0aa63460u},
    {0x92e87ceeu, 0xe431bc48u, 0x6f9c7aaau, 0x32f4287du, 0xeb924372u, 0x8260d1bcu, 0xbb97fec6u, 0x29c104dfu, 0x24aa4754u, 0x9a08a4ffu, 0x5c630eeau, 0x0e78ff20u},
    {0x96fb76cau, 0x92519ca9u, 0xa6ad99ccu, 0x3b0a1ec9u, 0x35cca96au, 0xe9400828u, 0xcc972cedu, 0x901598abu, 0x9194a48bu, 0xff891f51u, 0x1974e49eu, 0x152d8503u},
    {0xaaaf551au, 0x7f20be8eu, 0xaf38c3bfu, 0xeb250a6au, 0x4fed581bu, 0x4a4147fau, 0x21c097e3u, 0x2e57d55bu, 0x476dde9eu, 0x8b46b3d6u, 0x3ae1e53fu, 0x15cebb84u},
    {0xd26ebe58u, 0xfb73eaeau, 0x3de6a351u, 0x861c2369u, 0xf951c543u, 0x76e5bc3fu, 0x6a76590cu, 0xcc0868ceu, 0x35446d0bu, 0xf0a85a3fu, 0xa49a064fu, 0x0010a8c1u},
    {0x667bd107u, 0x42095dcau, 0x8731d905u, 0xb88e18a0u, 0xeb2d074bu, 0x4d9eaa70u, 0xe4790c93u, 0x9400c406u, 0xb8d714dfu, 0xb6b70a34u, 0x6d91387au, 0x07e3c51cu},
    {0x731e3ff8u, 0x26d6cf05u, 0x7b7c0273u, 0x1faec92du, 0x99363cf1u, 0x77badfa1u, 0x5e46429fu, 0x1be1b63fu, 0x1bf04296u, 0xfdebd05au, 0x3e898030u, 0x0916840au},
    {0x56be821cu, 0xdc435c2fu, 0xd228d866u, 0x238f84f9u, 0x776ffa2fu, 0x4574eaa5u, 0x8de35faeu, 0x7586a9d1u, 0x8476c66bu, 0x7b91fd87u, 0x67401cfbu, 0x17702f65u},
    {0x5a97350au, 0x8a7ba1b1u, 0x7197dea9u, 0x0c7e7432u, 0x64fb514fu, 0xbf0ee5adu, 0x25d59a08u, 0x8f272f54u, 0xb0ead8e5u, 0xe50279e5u, 0xf4608a4au, 0x0bedea03u},
    {0x5d9986a8u, 0x6791cb0fu, 0x364ceebau, 0xe329ef82u, 0x1ece2d85u, 0xa4eda9b0u, 0x50617381u, 0x88e2f0aau, 0x958b3000u, 0xb867f1c2u, 0x7967524eu, 0x083d38a0u},
    {0xcb89af51u, 0x1a2a5bf4u, 0xfbba7ca3u, 0xec71f13au, 0x32646160u, 0x71046590u, 0x8311a84du, 0x480a4a18u, 0x7ad91f53u, 0x6698e590u, 0x5d745072u, 0x08746207u},
    {0x9a1d2c25u, 0x3dc55103u, 0x57a98437u, 0xe8da66c8u, 0x13331128u, 0xb82e8f65u, 0x2a29ba38u, 0xb197b625u, 0xe32928cbu, 0x5dcbe4f4u, 0xf81f158cu, 0x0e91f80eu},
    {0x1c341746u, 0xf4df1f34u, 0x09d104f1u, 0x0a76e6a6u, 0x4c95b6d5u, 0x8de5476cu, 0x939d83c0u, 0x67eb88a9u, 0xb519952du, 0x9a793e85u, 0x92cae3aau, 0x11988fe5u},
    {0xa6b0fd59u, 0xd322c677u, 0x009687d4u, 0xddc76b07u, 0x60339eecu, 0x2745a8dfu, 0x5c9b2241u, 0xa8ea1b3du, 0x1814c738u, 0x5258e1cbu, 0x1327fd2fu, 0x0a513996u},
    {0xcd2dbfd7u, 0xfc8aa5c5u, 0xd26528c7u, 0x4874042cu, 0x232a8e28u, 0xd01b07fdu, 0x9b97e001u, 0x23d6a106u, 0x8b4c65b3u, 0xa1a742c3u, 0x27e00758u, 0x02050a15u},
    {0x9a0f8820u, 0xed6eb534u, 0x90d0d89eu, 0x8557e86fu, 0xa0de058cu, 0xdc405cbau, 0xadaa9f43u, 0x639892cdu, 0xff70e776u, 0xd659c27eu, 0xaf3c696bu, 0x0908ecb7u},
    {0xc5ce820fu, 0x075b3cd7u, 0x1c3edb0bu, 0x3ec6ba62u, 0x2bff6bceu, 0x168a13d8u, 0xf8c449d2u, 0x87663c4bu, 0xddc8d830u, 0x15f34c83u, 0x9caa2e85u, 0x0f9628b4u},
    {0xdb882f60u, 0xed6e6753u, 0x9db893eau, 0xd1849546u, 0x1ca4aac5u, 0x08715ae8u, 0xe0f61773u, 0x4c362c00u, 0x04dc9400u, 0x58e4b786u, 0xce28c06du, 0x041aad9au},
    {0x3b8e1ce7u, 0x9e2a2b80u, 0x701f5ab3u, 0xcede519du, 0x81ab4621u, 0xa0a6217eu, 0x9eee6510u, 0xde9fabafu, 0x8e4a8041u, 0xef148e59u, 0x3dff1a47u, 0x16ae3078u},
    {0x72ded94bu, 0x944a75c8u, 0x14d700cbu, 0x260dae75u, 0x68a854a2u, 0x7514a72du, 0x0387a395u, 0x3bb9c1d0u, 0x287aca8fu, 0xea4f0983u, 0xaf76e794u, 0x190d5914u},
    {0xa62b6c9du, 0x967d3988u, 0xa8eaff4eu, 0x4532383fu, 0x03310846u, 0x82383087u, 0xd396d7cfu, 0x15efebb5u, 0xee4e16bcu, 0xfab7cd07u, 0x884e56c4u, 0x02cb5d3au},
    {0xa653f6fcu, 0xe0c6a0c0u, 0x21bc8d58u, 0xc7a249dfu, 0x363665a0u, 0x74d9c6d4u, 0x2b6bf6ccu, 0x33c52549u, 0x887f8c8bu, 0x23c5935au, 0xa48f1eb6u, 0x1447c487u},
    {0x7dba9366u, 0x42b7fde3u, 0x27525bc3u, 0x7784894eu, 0xc1f5b1e9u, 0xb2b91b9du, 0xfcafb872u, 0x206f497du, 0x89a9b0bbu, 0x594137ccu, 0x20d7e399u, 0x0411cd9du},
    {0xa8e9b9afu, 0x44f6480eu, 0x766c8fe4u, 0xa96f7d65u, 0x28b540feu, 0xe82efd42u, 0xade53b2eu, 0x6723e5f0u, 0xfdd4230au, 0x25ff6eb6u, 0xef23c24au, 0x14c8ee06u},
    {0x0002fffdu, 0x76090000u, 0xc40c0002u, 0xebf4000bu, 0x53c758bau, 0x5f489857u, 0x70525745u, 0x77ce5853u, 0xa256ec6du, 0x5c071a97u, 0xfa80e493u, 0x15f65ec3u},
};
__device__ __constant__ static const uint32_t KINV_T2[32][12] = {
    {0x0002fffdu, 0x76090000u, 0xc40c0002u, 0xebf4000bu, 0x53c758bau, 0x5f489857u, 0x70525745u, 0x77ce5853u, 0xa256ec6du, 0x5c071a97u, 0xfa80e493u, 0x15f65ec3u},
    {0x00015554u, 0x18040000u, 0x3ab00001u, 0x85500005u, 0x253c276fu, 0x633cb57cu, 0x31ebb502u, 0x6e22d1ecu, 0xf2d14ca2u, 0xd3916126u, 0x1a006596u, 0x17fbb857u},
    {0x0000aaaau, 0x8c020000u, 0x9d580000u, 0xc2a80002u, 0x129e13b7u, 0x319e5abeu, 0x18f5da81u, 0x371168f6u, 0x7968a651u, 0x69c8b093u, 0x8d0032cbu, 0x0bfddc2bu},
    {0x00005555u, 0x46010000u, 0x4eac0000u, 0xe1540001u, 0x094f09dbu, 0x98cf2d5fu, 0x0c7aed40u, 0x9b88b47bu, 0xbcb45328u, 0xb4e45849u, 0xc6801965u, 0x05feee15u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x10000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x08000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x04000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x02000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x01000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00800000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00400000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00200000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00100000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00080000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00040000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00020000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00010000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00008000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00004000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00002000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00001000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000800u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000400u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000200u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000100u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000080u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000040u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000020u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000010u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000008u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000004u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000002u},
};

// 12-limb helpers on plain integers (not field elements).  Outputs are
// early-clobber: d may alias a or b, and every input word must be read before
// any output word is written.
__device__ __forceinline__ uint32_t limbs_sub(uint32_t* d, const uint32_t* a, const uint32_t* b)
{
    uint32_t borrow;
    asm("sub.cc.u32  %0, %13, %25;\n\t"
        "subc.cc.u32 %1, %14, %26;\n\t"
        "subc.cc.u32 %2, %15, %27;\n\t"
        "subc.cc.u32 %3, %16, %28;\n\t"
        "subc.cc.u32 %4, %17, %29;\n\t"
        "subc.cc.u32 %5, %18, %30;\n\t"
        "subc.cc.u32 %6, %19, %31;\n\t"
        "subc.cc.u32 %7, %20, %32;\n\t"
        "subc.cc.u32 %8, %21, %33;\n\t"
        "subc.cc.u32 %9, %22, %34;\n\t"
        "subc.cc.u32 %10, %23, %35;\n\t"
        "subc.cc.u32 %11, %24, %36;\n\t"
        "subc.u32    %12, 0, 0;"
        : "=&r"(d[0]), "=&r"(d[1]), "=&r"(d[2]), "=&r"(d[3]), "=&r"(d[4]), "=&r"(d[5]),
          "=&r"(d[6]), "=&r"(d[7]), "=&r"(d[8]), "=&r"(d[9]), "=&r"(d[10]), "=&r"(d[11]), "=&r"(borrow)
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]),
          "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]),
          "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]),
          "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]));
    return borrow;   // 0xffffffff if a < b
}

__device__ __forceinline__ void limbs_add(uint32_t* d, const uint32_t* a, const uint32_t* b)
{
    asm("add.cc.u32  %0, %12, %24;\n\t"
        "addc.cc.u32 %1, %13, %25;\n\t"
        "addc.cc.u32 %2, %14, %26;\n\t"
        "addc.cc.u32 %3, %15, %27;\n\t"
        "addc.cc.u32 %4, %16, %28;\n\t"
        "addc.cc.u32 %5, %17, %29;\n\t"
        "addc.cc.u32 %6, %18, %30;\n\t"
        "addc.cc.u32 %7, %19, %31;\n\t"
        "addc.cc.u32 %8, %20, %32;\n\t"
        "addc.cc.u32 %9, %21, %33;\n\t"
        "addc.cc.u32 %10, %22, %34;\n\t"
        "addc.u32    %11, %23, %35;"
        : "=&r"(d[0]), "=&r"(d[1]), "=&r"(d[2]), "=&r"(d[3]), "=&r"(d[4]), "=&r"(d[5]),
          "=&r"(d[6]), "=&r"(d[7]), "=&r"(d[8]), "=&r"(d[9]), "=&r"(d[10]), "=&r"(d[11])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]),
          "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]),
          "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]),
          "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]));
}

// r = a^-1 in Montgomery form for a in [0, 2p) (Montgomery form); zero maps
// to zero.  Branch-free per iteration (both differences are formed and one
// is selected), so lanes of a warp that invert different values stay
// converged until they finish; measured on GB300 this beat a branching form
// run by one lane per warp (66 against 89 microseconds per launch).
static __device__ __noinline__ fp fp_inv_vartime_call(const fp a)
{
    fp canon;
    fp_canon(canon, a);
    uint32_t u[12], v[12], r[12], s[12];
    uint32_t nz = 0;
#pragma unroll
    for (int i = 0; i < 12; i++) {
        u[i] = FP_P[i];
        v[i] = canon.v[i];
        r[i] = 0;
        s[i] = 0;
        nz |= canon.v[i];
    }
    fp out;
    fp_zero(out);
    if (nz == 0) return out;
    s[0] = 1;
    uint32_t k = 0;
    // strip v's trailing zeros (r = 0 stays 0)
    while (v[0] == 0) {
#pragma unroll
        for (int i = 0; i < 11; i++) v[i] = v[i + 1];
        v[11] = 0;
        k += 32;
    }
    {
        const uint32_t t = __ffs(v[0]) - 1;
        if (t) {
#pragma unroll
            for (int i = 0; i < 11; i++) v[i] = __funnelshift_r(v[i], v[i + 1], t);
            v[11] >>= t;
            k += t;
        }
    }
    for (int iter = 0; iter < 1024; iter++) {    // at most ~390 for 381-bit inputs
        uint32_t d1[12], d2[12];
        const uint32_t lt = limbs_sub(d1, u, v);          // u < v
        limbs_sub(d2, v, u);
        uint32_t z = 0;
#pragma unroll
        for (int i = 0; i < 12; i++) z |= d1[i];
        if (z == 0) {                                     // u == v == 1
            limbs_add(s, r, s);
#pragma unroll
            for (int i = 11; i > 0; i--) r[i] = __funnelshift_l(r[i - 1], r[i], 1);
            r[0] <<= 1;
            k += 1;
            break;
        }
        const bool gt = lt == 0;
        uint32_t w[12], sh[12], sum[12];
#pragma unroll
        for (int i = 0; i < 12; i++) {
            w[i] = gt ? d1[i] : d2[i];
            sh[i] = gt ? s[i] : r[i];
        }
        limbs_add(sum, r, s);
        // w is even and nonzero: w >>= t, sh <<= t
        while (w[0] == 0) {
#pragma unroll
            for (int i = 0; i < 11; i++) w[i] = w[i + 1];
            w[11] = 0;
#pragma unroll
            for (int i = 11; i > 0; i--) sh[i] = sh[i - 1];
            sh[0] = 0;
            k += 32;
        }
        const uint32_t t = __ffs(w[0]) - 1;
        if (t) {
#pragma unroll
            for (int i = 0; i < 11; i++) w[i] = __funnelshift_r(w[i], w[i + 1], t);
            w[11] >>= t;
#pragma unroll
            for (int i = 11; i > 0; i--) sh[i] = __funnelshift_l(sh[i - 1], sh[i], t);
            sh[0] <<= t;
        }
        k += t;
#pragma unroll
        for (int i = 0; i < 12; i++) {
            u[i] = gt ? w[i] : u[i];
            v[i] = gt ? v[i] : w[i];
            r[i] = gt ? sum[i] : sh[i];
            s[i] = gt ? sh[i] : sum[i];
        }
    }
    // r in [0, 2p]: reduce once, X = p - r
    uint32_t rr[12], pr[12];
    const uint32_t below = limbs_sub(rr, r, FP_P);        // r < p ?
#pragma unroll
    for (int i = 0; i < 12; i++) {
        pr[i] = FP_P[i];
        rr[i] = below ? r[i] : rr[i];
    }
    fp X;
    limbs_sub(X.v, pr, rr);
    const uint32_t ka = min(k >> 5, 24u), kb = k & 31;
    fp c1, c2;
#pragma unroll
    for (int i = 0; i < 12; i++) {
        c1.v[i] = KINV_T1[ka][i];
        c2.v[i] = KINV_T2[kb][i];
    }
    fp y;
    fp_mul(y, X, c1);
    fp_mul(out, y, c2);
    return out;
}

__device__ __forceinline__ void fp_inv_vartime(fp& r, const fp& a) { r = fp_inv_vartime_call(a); }

}  // namespace catmsm
