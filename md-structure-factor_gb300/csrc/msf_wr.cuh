// msf_wr.cuh -- w_R^k = exp(-2 pi i k / R), k < R, for the composite in-register
// radices of the mixed-radix FFT (msf_mixed.cuh): cos and sin of 2 pi k / R
// evaluated in FP64 and rounded to float, written out as literals by
// msf_wr_gen.py.  Every index is a compile-time constant once the DFT loops
// unroll, so these fold into immediates.
#pragma once

#include <cuda_runtime.h>

namespace msf {
namespace mixed {

template <int R> struct WR;

template <> struct WR<6> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 6) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.5f, -0.866025388f);
      case 2: return make_float2(-0.5f, -0.866025388f);
      case 3: return make_float2(-1.0f, -0.0f);
      case 4: return make_float2(-0.5f, 0.866025388f);
      case 5: return make_float2(0.5f, 0.866025388f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<9> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 9) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.766044438f, -0.642787635f);
      case 2: return make_float2(0.173648179f, -0.98480773f);
      case 3: return make_float2(-0.5f, -0.866025388f);
      case 4: return make_float2(-0.939692616f, -0.342020154f);
      case 5: return make_float2(-0.939692616f, 0.342020154f);
      case 6: return make_float2(-0.5f, 0.866025388f);
      case 7: return make_float2(0.173648179f, 0.98480773f);
      case 8: return make_float2(0.766044438f, 0.642787635f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<10> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 10) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.809017003f, -0.587785244f);
      case 2: return make_float2(0.309017003f, -0.95105654f);
      case 3: return make_float2(-0.309017003f, -0.95105654f);
      case 4: return make_float2(-0.809017003f, -0.587785244f);
      case 5: return make_float2(-1.0f, -0.0f);
      case 6: return make_float2(-0.809017003f, 0.587785244f);
      case 7: return make_float2(-0.309017003f, 0.95105654f);
      case 8: return make_float2(0.309017003f, 0.95105654f);
      case 9: return make_float2(0.809017003f, 0.587785244f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<12> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 12) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.866025388f, -0.5f);
      case 2: return make_float2(0.5f, -0.866025388f);
      case 3: return make_float2(0.0f, -1.0f);
      case 4: return make_float2(-0.5f, -0.866025388f);
      case 5: return make_float2(-0.866025388f, -0.5f);
      case 6: return make_float2(-1.0f, -0.0f);
      case 7: return make_float2(-0.866025388f, 0.5f);
      case 8: return make_float2(-0.5f, 0.866025388f);
      case 9: return make_float2(0.0f, 1.0f);
      case 10: return make_float2(0.5f, 0.866025388f);
      case 11: return make_float2(0.866025388f, 0.5f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<15> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 15) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.91354543f, -0.406736642f);
      case 2: return make_float2(0.669130623f, -0.74314481f);
      case 3: return make_float2(0.309017003f, -0.95105654f);
      case 4: return make_float2(-0.104528464f, -0.994521916f);
      case 5: return make_float2(-0.5f, -0.866025388f);
      case 6: return make_float2(-0.809017003f, -0.587785244f);
      case 7: return make_float2(-0.978147626f, -0.207911685f);
      case 8: return make_float2(-0.978147626f, 0.207911685f);
      case 9: return make_float2(-0.809017003f, 0.587785244f);
      case 10: return make_float2(-0.5f, 0.866025388f);
      case 11: return make_float2(-0.104528464f, 0.994521916f);
      case 12: return make_float2(0.309017003f, 0.95105654f);
      case 13: return make_float2(0.669130623f, 0.74314481f);
      case 14: return make_float2(0.91354543f, 0.406736642f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<18> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 18) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.939692616f, -0.342020154f);
      case 2: return make_float2(0.766044438f, -0.642787635f);
      case 3: return make_float2(0.5f, -0.866025388f);
      case 4: return make_float2(0.173648179f, -0.98480773f);
      case 5: return make_float2(-0.173648179f, -0.98480773f);
      case 6: return make_float2(-0.5f, -0.866025388f);
      case 7: return make_float2(-0.766044438f, -0.642787635f);
      case 8: return make_float2(-0.939692616f, -0.342020154f);
      case 9: return make_float2(-1.0f, -0.0f);
      case 10: return make_float2(-0.939692616f, 0.342020154f);
      case 11: return make_float2(-0.766044438f, 0.642787635f);
      case 12: return make_float2(-0.5f, 0.866025388f);
      case 13: return make_float2(-0.173648179f, 0.98480773f);
      case 14: return make_float2(0.173648179f, 0.98480773f);
      case 15: return make_float2(0.5f, 0.866025388f);
      case 16: return make_float2(0.766044438f, 0.642787635f);
      case 17: return make_float2(0.939692616f, 0.342020154f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<20> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 20) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.95105654f, -0.309017003f);
      case 2: return make_float2(0.809017003f, -0.587785244f);
      case 3: return make_float2(0.587785244f, -0.809017003f);
      case 4: return make_float2(0.309017003f, -0.95105654f);
      case 5: return make_float2(0.0f, -1.0f);
      case 6: return make_float2(-0.309017003f, -0.95105654f);
      case 7: return make_float2(-0.587785244f, -0.809017003f);
      case 8: return make_float2(-0.809017003f, -0.587785244f);
      case 9: return make_float2(-0.95105654f, -0.309017003f);
      case 10: return make_float2(-1.0f, -0.0f);
      case 11: return make_float2(-0.95105654f, 0.309017003f);
      case 12: return make_float2(-0.809017003f, 0.587785244f);
      case 13: return make_float2(-0.587785244f, 0.809017003f);
      case 14: return make_float2(-0.309017003f, 0.95105654f);
      case 15: return make_float2(0.0f, 1.0f);
      case 16: return make_float2(0.309017003f, 0.95105654f);
      case 17: return make_float2(0.587785244f, 0.809017003f);
      case 18: return make_float2(0.809017003f, 0.587785244f);
      case 19: return make_float2(0.95105654f, 0.309017003f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<25> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 25) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.968583167f, -0.24868989f);
      case 2: return make_float2(0.876306653f, -0.481753677f);
      case 3: return make_float2(0.72896862f, -0.684547126f);
      case 4: return make_float2(0.535826802f, -0.844327927f);
      case 5: return make_float2(0.309017003f, -0.95105654f);
      case 6: return make_float2(0.0627905205f, -0.998026729f);
      case 7: return make_float2(-0.187381312f, -0.982287228f);
      case 8: return make_float2(-0.425779283f, -0.904827058f);
      case 9: return make_float2(-0.637423992f, -0.770513237f);
      case 10: return make_float2(-0.809017003f, -0.587785244f);
      case 11: return make_float2(-0.92977649f, -0.368124545f);
      case 12: return make_float2(-0.992114723f, -0.125333235f);
      case 13: return make_float2(-0.992114723f, 0.125333235f);
      case 14: return make_float2(-0.92977649f, 0.368124545f);
      case 15: return make_float2(-0.809017003f, 0.587785244f);
      case 16: return make_float2(-0.637423992f, 0.770513237f);
      case 17: return make_float2(-0.425779283f, 0.904827058f);
      case 18: return make_float2(-0.187381312f, 0.982287228f);
      case 19: return make_float2(0.0627905205f, 0.998026729f);
      case 20: return make_float2(0.309017003f, 0.95105654f);
      case 21: return make_float2(0.535826802f, 0.844327927f);
      case 22: return make_float2(0.72896862f, 0.684547126f);
      case 23: return make_float2(0.876306653f, 0.481753677f);
      case 24: return make_float2(0.968583167f, 0.24868989f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

template <> struct WR<27> {
  static __host__ __device__ constexpr float2 w(int k) {
    switch (k % 27) {
      case 0: return make_float2(1.0f, -0.0f);
      case 1: return make_float2(0.973044872f, -0.230615869f);
      case 2: return make_float2(0.89363265f, -0.448799193f);
      case 3: return make_float2(0.766044438f, -0.642787635f);
      case 4: return make_float2(0.597158611f, -0.802123189f);
      case 5: return make_float2(0.396079779f, -0.918216109f);
      case 6: return make_float2(0.173648179f, -0.98480773f);
      case 7: return make_float2(-0.0581448302f, -0.998308182f);
      case 8: return make_float2(-0.286803246f, -0.957989514f);
      case 9: return make_float2(-0.5f, -0.866025388f);
      case 10: return make_float2(-0.686241627f, -0.72737366f);
      case 11: return make_float2(-0.835487783f, -0.549508989f);
      case 12: return make_float2(-0.939692616f, -0.342020154f);
      case 13: return make_float2(-0.99323833f, -0.116092913f);
      case 14: return make_float2(-0.99323833f, 0.116092913f);
      case 15: return make_float2(-0.939692616f, 0.342020154f);
      case 16: return make_float2(-0.835487783f, 0.549508989f);
      case 17: return make_float2(-0.686241627f, 0.72737366f);
      case 18: return make_float2(-0.5f, 0.866025388f);
      case 19: return make_float2(-0.286803246f, 0.957989514f);
      case 20: return make_float2(-0.0581448302f, 0.998308182f);
      case 21: return make_float2(0.173648179f, 0.98480773f);
      case 22: return make_float2(0.396079779f, 0.918216109f);
      case 23: return make_float2(0.597158611f, 0.802123189f);
      case 24: return make_float2(0.766044438f, 0.642787635f);
      case 25: return make_float2(0.89363265f, 0.448799193f);
      case 26: return make_float2(0.973044872f, 0.230615869f);
    }
    return make_float2(1.0f, 0.0f);
  }
};

}  // namespace mixed
}  // namespace msf
