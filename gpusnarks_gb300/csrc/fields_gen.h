// Generated by gpusnarks_gb300/gen_fields.py from gpusnarks_gb300/fields.py.
// Do not edit by hand.
#pragma once
#include <cstdint>

#include "gsn_compat.h"

namespace gsn {

// p32: 32-bit modulus, 1 limb(s), 2-adicity 30, generator 5
struct FieldP32 {
  static constexpr int ID = 0;
  static constexpr int N = 1;
  static constexpr uint32_t PINV = 0xBFFFFFFFu;
  static constexpr int TWO_ADICITY = 30;
  static constexpr uint32_t GENERATOR = 5u;
  static constexpr int BITS = 32;
  // floor(R / p): 1 means no headroom, >= 4 allows sums of two [0,2p) values.
  static constexpr uint32_t HEADROOM = 1u;
  __host__ __device__ static constexpr uint32_t mod(int i) {
    switch (i) {
      case 0: return 0xC0000001u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r1(int i) {
    switch (i) {
      case 0: return 0x3FFFFFFFu;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r2(int i) {
    switch (i) {
      case 0: return 0x6AAAAAADu;
      default: return 0u;
    }
  }

};

// bls12_381_fr: 255-bit modulus, 8 limb(s), 2-adicity 32, generator 7
struct FieldBLS12_381 {
  static constexpr int ID = 1;
  static constexpr int N = 8;
  static constexpr uint32_t PINV = 0xFFFFFFFFu;
  static constexpr int TWO_ADICITY = 32;
  static constexpr uint32_t GENERATOR = 7u;
  static constexpr int BITS = 255;
  // floor(R / p): 1 means no headroom, >= 4 allows sums of two [0,2p) values.
  static constexpr uint32_t HEADROOM = 2u;
  __host__ __device__ static constexpr uint32_t mod(int i) {
    switch (i) {
      case 0: return 0x00000001u;
      case 1: return 0xFFFFFFFFu;
      case 2: return 0xFFFE5BFEu;
      case 3: return 0x53BDA402u;
      case 4: return 0x09A1D805u;
      case 5: return 0x3339D808u;
      case 6: return 0x299D7D48u;
      case 7: return 0x73EDA753u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r1(int i) {
    switch (i) {
      case 0: return 0xFFFFFFFEu;
      case 1: return 0x00000001u;
      case 2: return 0x00034802u;
      case 3: return 0x5884B7FAu;
      case 4: return 0xECBC4FF5u;
      case 5: return 0x998C4FEFu;
      case 6: return 0xACC5056Fu;
      case 7: return 0x1824B159u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r2(int i) {
    switch (i) {
      case 0: return 0xF3F29C6Du;
      case 1: return 0xC999E990u;
      case 2: return 0x87925C23u;
      case 3: return 0x2B6CEDCBu;
      case 4: return 0x7254398Fu;
      case 5: return 0x05D31496u;
      case 6: return 0x9F59FF11u;
      case 7: return 0x0748D9D9u;
      default: return 0u;
    }
  }

};

// mnt4753_fr: 753-bit modulus, 24 limb(s), 2-adicity 30, generator 11
struct FieldMNT4_753 {
  static constexpr int ID = 2;
  static constexpr int N = 24;
  static constexpr uint32_t PINV = 0x3FFFFFFFu;
  static constexpr int TWO_ADICITY = 30;
  static constexpr uint32_t GENERATOR = 11u;
  static constexpr int BITS = 753;
  // floor(R / p): 1 means no headroom, >= 4 allows sums of two [0,2p) values.
  static constexpr uint32_t HEADROOM = 37054u;
  __host__ __device__ static constexpr uint32_t mod(int i) {
    switch (i) {
      case 0: return 0x40000001u;
      case 1: return 0xD90776E2u;
      case 2: return 0x0FA13A4Fu;
      case 3: return 0x4EA09917u;
      case 4: return 0x3F005797u;
      case 5: return 0xD6C381BCu;
      case 6: return 0x34993AA4u;
      case 7: return 0xB9DFF976u;
      case 8: return 0x29212636u;
      case 9: return 0x3EEBCA94u;
      case 10: return 0xC859A99Bu;
      case 11: return 0xB26C5C28u;
      case 12: return 0xA15AF79Du;
      case 13: return 0x99D124D9u;
      case 14: return 0xE8A0ED8Du;
      case 15: return 0x07FDB925u;
      case 16: return 0x6C97D873u;
      case 17: return 0x5EB7E8F9u;
      case 18: return 0x5B8FAFEDu;
      case 19: return 0xB7F99750u;
      case 20: return 0xEEE2CDADu;
      case 21: return 0x10229022u;
      case 22: return 0x2D92C411u;
      case 23: return 0x0001C4C6u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r1(int i) {
    switch (i) {
      case 0: return 0x7FFF6F42u;
      case 1: return 0xB9968014u;
      case 2: return 0xB589CEA8u;
      case 3: return 0x4EB16817u;
      case 4: return 0x0C79E179u;
      case 5: return 0xA1EBD2D9u;
      case 6: return 0xC549C0DAu;
      case 7: return 0x0F725CAEu;
      case 8: return 0xD3E6DAD4u;
      case 9: return 0xAB0C4EE6u;
      case 10: return 0xDE0CCB62u;
      case 11: return 0x9FBCA908u;
      case 12: return 0x13338498u;
      case 13: return 0x320C3BB7u;
      case 14: return 0xD2F00A62u;
      case 15: return 0x598B4302u;
      case 16: return 0xFD8CA621u;
      case 17: return 0x4074C9CBu;
      case 18: return 0x3865E88Cu;
      case 19: return 0x0FA47EDBu;
      case 20: return 0x1FF9A195u;
      case 21: return 0x95455FB3u;
      case 22: return 0x9EC8E242u;
      case 23: return 0x00007B47u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r2(int i) {
    switch (i) {
      case 0: return 0xB7F4C8D1u;
      case 1: return 0x3F9C69C7u;
      case 2: return 0xEE48D127u;
      case 3: return 0x70A50FA9u;
      case 4: return 0x009569CBu;
      case 5: return 0xCDBE6702u;
      case 6: return 0xC49EDC38u;
      case 7: return 0x6BD8C6C6u;
      case 8: return 0xC35EE94Eu;
      case 9: return 0x7955876Cu;
      case 10: return 0xBE54A3F4u;
      case 11: return 0xC7285529u;
      case 12: return 0xECEC77CFu;
      case 13: return 0xDED52121u;
      case 14: return 0xEE12EE8Eu;
      case 15: return 0x99BE80F2u;
      case 16: return 0x493BDCEFu;
      case 17: return 0xC8A0FF01u;
      case 18: return 0xF3D9A316u;
      case 19: return 0xACC27988u;
      case 20: return 0xFB44B3C9u;
      case 21: return 0xD9E817A8u;
      case 22: return 0x8037E0E4u;
      case 23: return 0x000005B5u;
      default: return 0u;
    }
  }

};

// mnt4753_fq: 753-bit modulus, 24 limb(s), 2-adicity 15, generator 13
struct FieldMNT4_753_Q {
  static constexpr int ID = 3;
  static constexpr int N = 24;
  static constexpr uint32_t PINV = 0xE45E7FFFu;
  static constexpr int TWO_ADICITY = 15;
  static constexpr uint32_t GENERATOR = 13u;
  static constexpr int BITS = 753;
  // floor(R / p): 1 means no headroom, >= 4 allows sums of two [0,2p) values.
  static constexpr uint32_t HEADROOM = 37054u;
  __host__ __device__ static constexpr uint32_t mod(int i) {
    switch (i) {
      case 0: return 0x245E8001u;
      case 1: return 0x5E9063DEu;
      case 2: return 0x2CDD119Fu;
      case 3: return 0xE39D5452u;
      case 4: return 0x9AC425F0u;
      case 5: return 0x63881071u;
      case 6: return 0x767254A4u;
      case 7: return 0x685ACCE9u;
      case 8: return 0xCB537E38u;
      case 9: return 0xB80F0DA5u;
      case 10: return 0xF218059Du;
      case 11: return 0xB117E776u;
      case 12: return 0xA15AF79Du;
      case 13: return 0x99D124D9u;
      case 14: return 0xE8A0ED8Du;
      case 15: return 0x07FDB925u;
      case 16: return 0x6C97D873u;
      case 17: return 0x5EB7E8F9u;
      case 18: return 0x5B8FAFEDu;
      case 19: return 0xB7F99750u;
      case 20: return 0xEEE2CDADu;
      case 21: return 0x10229022u;
      case 22: return 0x2D92C411u;
      case 23: return 0x0001C4C6u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r1(int i) {
    switch (i) {
      case 0: return 0xD9DC6F42u;
      case 1: return 0x98A8ECABu;
      case 2: return 0x5A034686u;
      case 3: return 0x91CD31C6u;
      case 4: return 0xCD14572Eu;
      case 5: return 0x97C3E4A0u;
      case 6: return 0xC788B601u;
      case 7: return 0x79589819u;
      case 8: return 0x2108976Fu;
      case 9: return 0xED269C94u;
      case 10: return 0xCF031D68u;
      case 11: return 0x1E0F4D8Au;
      case 12: return 0x13338559u;
      case 13: return 0x320C3BB7u;
      case 14: return 0xD2F00A62u;
      case 15: return 0x598B4302u;
      case 16: return 0xFD8CA621u;
      case 17: return 0x4074C9CBu;
      case 18: return 0x3865E88Cu;
      case 19: return 0x0FA47EDBu;
      case 20: return 0x1FF9A195u;
      case 21: return 0x95455FB3u;
      case 22: return 0x9EC8E242u;
      case 23: return 0x00007B47u;
      default: return 0u;
    }
  }

  __host__ __device__ static constexpr uint32_t r2(int i) {
    switch (i) {
      case 0: return 0xCFD190C8u;
      case 1: return 0x84717088u;
      case 2: return 0x7DF03C0Au;
      case 3: return 0xC7D9FF8Eu;
      case 4: return 0x242B3507u;
      case 5: return 0xA24BEA56u;
      case 6: return 0xA0714C7Du;
      case 7: return 0xA896A656u;
      case 8: return 0xFF6F3DDFu;
      case 9: return 0x80A46659u;
      case 10: return 0xF88D7CE8u;
      case 11: return 0x2F47839Eu;
      case 12: return 0x04A3B597u;
      case 13: return 0xA8C86D46u;
      case 14: return 0xC4F7EF07u;
      case 15: return 0xE03C79CAu;
      case 16: return 0xF4A81245u;
      case 17: return 0x2505DAF1u;
      case 18: return 0x4C381723u;
      case 19: return 0x8E460575u;
      case 20: return 0xCBFDACAFu;
      case 21: return 0xB081F15Bu;
      case 22: return 0xE89CB485u;
      case 23: return 0x00002A33u;
      default: return 0u;
    }
  }

};

}  // namespace gsn
