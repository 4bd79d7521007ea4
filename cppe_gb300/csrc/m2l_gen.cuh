// Generated by gen_m2l.py -- do not edit.
#pragma once

// M2L, source order 1, expansion order 5: Msize 55, Lsize 35
template <typename T>
__device__ __forceinline__ void m2l_m1_p5(T x, T y, T z, const T* __restrict__ Mb, T* __restrict__ acc) {
  const T r2 = x * x + y * y + z * z;
  const T ir2 = T(1) / r2;
  const T D0 = rsqrt_t(r2);
  const T D1 = -(T(1) * (x * D0)) * ir2 * cinv<T>(1);
  const T D2 = -(T(1) * (y * D0)) * ir2 * cinv<T>(1);
  const T D3 = -(T(1) * (z * D0)) * ir2 * cinv<T>(1);
  const T D4 = -(T(3) * (T(2) * x * D1) + T(1) * (T(2) * D0)) * ir2 * cinv<T>(2);
  const T D5 = -(T(3) * (x * D2 + y * D1)) * ir2 * cinv<T>(2);
  const T D6 = -(T(3) * (x * D3 + z * D1)) * ir2 * cinv<T>(2);
  const T D7 = -(T(3) * (T(2) * y * D2) + T(1) * (T(2) * D0)) * ir2 * cinv<T>(2);
  const T D8 = -(T(3) * (y * D3 + z * D2)) * ir2 * cinv<T>(2);
  const T D9 = -(T(3) * (T(2) * z * D3) + T(1) * (T(2) * D0)) * ir2 * cinv<T>(2);
  const T D10 = -(T(5) * (T(3) * x * D4) + T(2) * (T(6) * D1)) * ir2 * cinv<T>(3);
  const T D11 = -(T(5) * (T(2) * x * D5 + y * D4) + T(2) * (T(2) * D2)) * ir2 * cinv<T>(3);
  const T D12 = -(T(5) * (T(2) * x * D6 + z * D4) + T(2) * (T(2) * D3)) * ir2 * cinv<T>(3);
  const T D13 = -(T(5) * (x * D7 + T(2) * y * D5) + T(2) * (T(2) * D1)) * ir2 * cinv<T>(3);
  const T D14 = -(T(5) * (x * D8 + y * D6 + z * D5)) * ir2 * cinv<T>(3);
  const T D15 = -(T(5) * (x * D9 + T(2) * z * D6) + T(2) * (T(2) * D1)) * ir2 * cinv<T>(3);
  const T D16 = -(T(5) * (T(3) * y * D7) + T(2) * (T(6) * D2)) * ir2 * cinv<T>(3);
  const T D17 = -(T(5) * (T(2) * y * D8 + z * D7) + T(2) * (T(2) * D3)) * ir2 * cinv<T>(3);
  const T D18 = -(T(5) * (y * D9 + T(2) * z * D8) + T(2) * (T(2) * D2)) * ir2 * cinv<T>(3);
  const T D19 = -(T(5) * (T(3) * z * D9) + T(2) * (T(6) * D3)) * ir2 * cinv<T>(3);
  const T D20 = -(T(7) * (T(4) * x * D10) + T(3) * (T(12) * D4)) * ir2 * cinv<T>(4);
  const T D21 = -(T(7) * (T(3) * x * D11 + y * D10) + T(3) * (T(6) * D5)) * ir2 * cinv<T>(4);
  const T D22 = -(T(7) * (T(3) * x * D12 + z * D10) + T(3) * (T(6) * D6)) * ir2 * cinv<T>(4);
  const T D23 = -(T(7) * (T(2) * x * D13 + T(2) * y * D11) + T(3) * (T(2) * D7 + T(2) * D4)) * ir2 * cinv<T>(4);
  const T D24 = -(T(7) * (T(2) * x * D14 + y * D12 + z * D11) + T(3) * (T(2) * D8)) * ir2 * cinv<T>(4);
  const T D25 = -(T(7) * (T(2) * x * D15 + T(2) * z * D12) + T(3) * (T(2) * D9 + T(2) * D4)) * ir2 * cinv<T>(4);
  const T D26 = -(T(7) * (x * D16 + T(3) * y * D13) + T(3) * (T(6) * D5)) * ir2 * cinv<T>(4);
  const T D27 = -(T(7) * (x * D17 + T(2) * y * D14 + z * D13) + T(3) * (T(2) * D6)) * ir2 * cinv<T>(4);
  const T D28 = -(T(7) * (x * D18 + y * D15 + T(2) * z * D14) + T(3) * (T(2) * D5)) * ir2 * cinv<T>(4);
  const T D29 = -(T(7) * (x * D19 + T(3) * z * D15) + T(3) * (T(6) * D6)) * ir2 * cinv<T>(4);
  const T D30 = -(T(7) * (T(4) * y * D16) + T(3) * (T(12) * D7)) * ir2 * cinv<T>(4);
  const T D31 = -(T(7) * (T(3) * y * D17 + z * D16) + T(3) * (T(6) * D8)) * ir2 * cinv<T>(4);
  const T D32 = -(T(7) * (T(2) * y * D18 + T(2) * z * D17) + T(3) * (T(2) * D9 + T(2) * D7)) * ir2 * cinv<T>(4);
  const T D33 = -(T(7) * (y * D19 + T(3) * z * D18) + T(3) * (T(6) * D8)) * ir2 * cinv<T>(4);
  const T D34 = -(T(7) * (T(4) * z * D19) + T(3) * (T(12) * D9)) * ir2 * cinv<T>(4);
  const T D35 = -(T(9) * (T(5) * x * D20) + T(4) * (T(20) * D10)) * ir2 * cinv<T>(5);
  const T D36 = -(T(9) * (T(4) * x * D21 + y * D20) + T(4) * (T(12) * D11)) * ir2 * cinv<T>(5);
  const T D37 = -(T(9) * (T(4) * x * D22 + z * D20) + T(4) * (T(12) * D12)) * ir2 * cinv<T>(5);
  const T D38 = -(T(9) * (T(3) * x * D23 + T(2) * y * D21) + T(4) * (T(6) * D13 + T(2) * D10)) * ir2 * cinv<T>(5);
  const T D39 = -(T(9) * (T(3) * x * D24 + y * D22 + z * D21) + T(4) * (T(6) * D14)) * ir2 * cinv<T>(5);
  const T D40 = -(T(9) * (T(3) * x * D25 + T(2) * z * D22) + T(4) * (T(6) * D15 + T(2) * D10)) * ir2 * cinv<T>(5);
  const T D41 = -(T(9) * (T(2) * x * D26 + T(3) * y * D23) + T(4) * (T(2) * D16 + T(6) * D11)) * ir2 * cinv<T>(5);
  const T D42 = -(T(9) * (T(2) * x * D27 + T(2) * y * D24 + z * D23) + T(4) * (T(2) * D17 + T(2) * D12)) * ir2 * cinv<T>(5);
  const T D43 = -(T(9) * (T(2) * x * D28 + y * D25 + T(2) * z * D24) + T(4) * (T(2) * D18 + T(2) * D11)) * ir2 * cinv<T>(5);
  const T D44 = -(T(9) * (T(2) * x * D29 + T(3) * z * D25) + T(4) * (T(2) * D19 + T(6) * D12)) * ir2 * cinv<T>(5);
  const T D45 = -(T(9) * (x * D30 + T(4) * y * D26) + T(4) * (T(12) * D13)) * ir2 * cinv<T>(5);
  const T D46 = -(T(9) * (x * D31 + T(3) * y * D27 + z * D26) + T(4) * (T(6) * D14)) * ir2 * cinv<T>(5);
  const T D47 = -(T(9) * (x * D32 + T(2) * y * D28 + T(2) * z * D27) + T(4) * (T(2) * D15 + T(2) * D13)) * ir2 * cinv<T>(5);
  const T D48 = -(T(9) * (x * D33 + y * D29 + T(3) * z * D28) + T(4) * (T(6) * D14)) * ir2 * cinv<T>(5);
  const T D49 = -(T(9) * (x * D34 + T(4) * z * D29) + T(4) * (T(12) * D15)) * ir2 * cinv<T>(5);
  const T D50 = -(T(9) * (T(5) * y * D30) + T(4) * (T(20) * D16)) * ir2 * cinv<T>(5);
  const T D51 = -(T(9) * (T(4) * y * D31 + z * D30) + T(4) * (T(12) * D17)) * ir2 * cinv<T>(5);
  const T D52 = -(T(9) * (T(3) * y * D32 + T(2) * z * D31) + T(4) * (T(6) * D18 + T(2) * D16)) * ir2 * cinv<T>(5);
  const T D53 = -(T(9) * (T(2) * y * D33 + T(3) * z * D32) + T(4) * (T(2) * D19 + T(6) * D17)) * ir2 * cinv<T>(5);
  const T D54 = -(T(9) * (y * D34 + T(4) * z * D33) + T(4) * (T(12) * D18)) * ir2 * cinv<T>(5);
  const T D55 = -(T(9) * (T(5) * z * D34) + T(4) * (T(20) * D19)) * ir2 * cinv<T>(5);
  { const T mk = Mb[0];
    acc[0] = fma(D1, mk, acc[0]);
    acc[1] = fma(D4, mk, acc[1]);
    acc[2] = fma(D5, mk, acc[2]);
    acc[3] = fma(D6, mk, acc[3]);
    acc[4] = fma(D10, mk, acc[4]);
    acc[5] = fma(D11, mk, acc[5]);
    acc[6] = fma(D12, mk, acc[6]);
    acc[7] = fma(D13, mk, acc[7]);
    acc[8] = fma(D14, mk, acc[8]);
    acc[9] = fma(D15, mk, acc[9]);
    acc[10] = fma(D20, mk, acc[10]);
    acc[11] = fma(D21, mk, acc[11]);
    acc[12] = fma(D22, mk, acc[12]);
    acc[13] = fma(D23, mk, acc[13]);
    acc[14] = fma(D24, mk, acc[14]);
    acc[15] = fma(D25, mk, acc[15]);
    acc[16] = fma(D26, mk, acc[16]);
    acc[17] = fma(D27, mk, acc[17]);
    acc[18] = fma(D28, mk, acc[18]);
    acc[19] = fma(D29, mk, acc[19]);
    acc[20] = fma(D35, mk, acc[20]);
    acc[21] = fma(D36, mk, acc[21]);
    acc[22] = fma(D37, mk, acc[22]);
    acc[23] = fma(D38, mk, acc[23]);
    acc[24] = fma(D39, mk, acc[24]);
    acc[25] = fma(D40, mk, acc[25]);
    acc[26] = fma(D41, mk, acc[26]);
    acc[27] = fma(D42, mk, acc[27]);
    acc[28] = fma(D43, mk, acc[28]);
    acc[29] = fma(D44, mk, acc[29]);
    acc[30] = fma(D45, mk, acc[30]);
    acc[31] = fma(D46, mk, acc[31]);
    acc[32] = fma(D47, mk, acc[32]);
    acc[33] = fma(D48, mk, acc[33]);
    acc[34] = fma(D49, mk, acc[34]);
  }
  { const T mk = Mb[1];
    acc[0] = fma(D2, mk, acc[0]);
    acc[1] = fma(D5, mk, acc[1]);
    acc[2] = fma(D7, mk, acc[2]);
    acc[3] = fma(D8, mk, acc[3]);
    acc[4] = fma(D11, mk, acc[4]);
    acc[5] = fma(D13, mk, acc[5]);
    acc[6] = fma(D14, mk, acc[6]);
    acc[7] = fma(D16, mk, acc[7]);
    acc[8] = fma(D17, mk, acc[8]);
    acc[9] = fma(D18, mk, acc[9]);
    acc[10] = fma(D21, mk, acc[10]);
    acc[11] = fma(D23, mk, acc[11]);
    acc[12] = fma(D24, mk, acc[12]);
    acc[13] = fma(D26, mk, acc[13]);
    acc[14] = fma(D27, mk, acc[14]);
    acc[15] = fma(D28, mk, acc[15]);
    acc[16] = fma(D30, mk, acc[16]);
    acc[17] = fma(D31, mk, acc[17]);
    acc[18] = fma(D32, mk, acc[18]);
    acc[19] = fma(D33, mk, acc[19]);
    acc[20] = fma(D36, mk, acc[20]);
    acc[21] = fma(D38, mk, acc[21]);
    acc[22] = fma(D39, mk, acc[22]);
    acc[23] = fma(D41, mk, acc[23]);
    acc[24] = fma(D42, mk, acc[24]);
    acc[25] = fma(D43, mk, acc[25]);
    acc[26] = fma(D45, mk, acc[26]);
    acc[27] = fma(D46, mk, acc[27]);
    acc[28] = fma(D47, mk, acc[28]);
    acc[29] = fma(D48, mk, acc[29]);
    acc[30] = fma(D50, mk, acc[30]);
    acc[31] = fma(D51, mk, acc[31]);
    acc[32] = fma(D52, mk, acc[32]);
    acc[33] = fma(D53, mk, acc[33]);
    acc[34] = fma(D54, mk, acc[34]);
  }
  { const T mk = Mb[2];
    acc[0] = fma(D3, mk, acc[0]);
    acc[1] = fma(D6, mk, acc[1]);
    acc[2] = fma(D8, mk, acc[2]);
    acc[3] = fma(D9, mk, acc[3]);
    acc[4] = fma(D12, mk, acc[4]);
    acc[5] = fma(D14, mk, acc[5]);
    acc[6] = fma(D15, mk, acc[6]);
    acc[7] = fma(D17, mk, acc[7]);
    acc[8] = fma(D18, mk, acc[8]);
    acc[9] = fma(D19, mk, acc[9]);
    acc[10] = fma(D22, mk, acc[10]);
    acc[11] = fma(D24, mk, acc[11]);
    acc[12] = fma(D25, mk, acc[12]);
    acc[13] = fma(D27, mk, acc[13]);
    acc[14] = fma(D28, mk, acc[14]);
    acc[15] = fma(D29, mk, acc[15]);
    acc[16] = fma(D31, mk, acc[16]);
    acc[17] = fma(D32, mk, acc[17]);
    acc[18] = fma(D33, mk, acc[18]);
    acc[19] = fma(D34, mk, acc[19]);
    acc[20] = fma(D37, mk, acc[20]);
    acc[21] = fma(D39, mk, acc[21]);
    acc[22] = fma(D40, mk, acc[22]);
    acc[23] = fma(D42, mk, acc[23]);
    acc[24] = fma(D43, mk, acc[24]);
    acc[25] = fma(D44, mk, acc[25]);
    acc[26] = fma(D46, mk, acc[26]);
    acc[27] = fma(D47, mk, acc[27]);
    acc[28] = fma(D48, mk, acc[28]);
    acc[29] = fma(D49, mk, acc[29]);
    acc[30] = fma(D51, mk, acc[30]);
    acc[31] = fma(D52, mk, acc[31]);
    acc[32] = fma(D53, mk, acc[32]);
    acc[33] = fma(D54, mk, acc[33]);
    acc[34] = fma(D55, mk, acc[34]);
  }
  { const T mk = Mb[3];
    acc[0] = fma(D4, mk, acc[0]);
    acc[1] = fma(D10, mk, acc[1]);
    acc[2] = fma(D11, mk, acc[2]);
    acc[3] = fma(D12, mk, acc[3]);
    acc[4] = fma(D20, mk, acc[4]);
    acc[5] = fma(D21, mk, acc[5]);
    acc[6] = fma(D22, mk, acc[6]);
    acc[7] = fma(D23, mk, acc[7]);
    acc[8] = fma(D24, mk, acc[8]);
    acc[9] = fma(D25, mk, acc[9]);
    acc[10] = fma(D35, mk, acc[10]);
    acc[11] = fma(D36, mk, acc[11]);
    acc[12] = fma(D37, mk, acc[12]);
    acc[13] = fma(D38, mk, acc[13]);
    acc[14] = fma(D39, mk, acc[14]);
    acc[15] = fma(D40, mk, acc[15]);
    acc[16] = fma(D41, mk, acc[16]);
    acc[17] = fma(D42, mk, acc[17]);
    acc[18] = fma(D43, mk, acc[18]);
    acc[19] = fma(D44, mk, acc[19]);
  }
  { const T mk = Mb[4];
    acc[0] = fma(D5, mk, acc[0]);
    acc[1] = fma(D11, mk, acc[1]);
    acc[2] = fma(D13, mk, acc[2]);
    acc[3] = fma(D14, mk, acc[3]);
    acc[4] = fma(D21, mk, acc[4]);
    acc[5] = fma(D23, mk, acc[5]);
    acc[6] = fma(D24, mk, acc[6]);
    acc[7] = fma(D26, mk, acc[7]);
    acc[8] = fma(D27, mk, acc[8]);
    acc[9] = fma(D28, mk, acc[9]);
    acc[10] = fma(D36, mk, acc[10]);
    acc[11] = fma(D38, mk, acc[11]);
    acc[12] = fma(D39, mk, acc[12]);
    acc[13] = fma(D41, mk, acc[13]);
    acc[14] = fma(D42, mk, acc[14]);
    acc[15] = fma(D43, mk, acc[15]);
    acc[16] = fma(D45, mk, acc[16]);
    acc[17] = fma(D46, mk, acc[17]);
    acc[18] = fma(D47, mk, acc[18]);
    acc[19] = fma(D48, mk, acc[19]);
  }
  { const T mk = Mb[5];
    acc[0] = fma(D6, mk, acc[0]);
    acc[1] = fma(D12, mk, acc[1]);
    acc[2] = fma(D14, mk, acc[2]);
    acc[3] = fma(D15, mk, acc[3]);
    acc[4] = fma(D22, mk, acc[4]);
    acc[5] = fma(D24, mk, acc[5]);
    acc[6] = fma(D25, mk, acc[6]);
    acc[7] = fma(D27, mk, acc[7]);
    acc[8] = fma(D28, mk, acc[8]);
    acc[9] = fma(D29, mk, acc[9]);
    acc[10] = fma(D37, mk, acc[10]);
    acc[11] = fma(D39, mk, acc[11]);
    acc[12] = fma(D40, mk, acc[12]);
    acc[13] = fma(D42, mk, acc[13]);
    acc[14] = fma(D43, mk, acc[14]);
    acc[15] = fma(D44, mk, acc[15]);
    acc[16] = fma(D46, mk, acc[16]);
    acc[17] = fma(D47, mk, acc[17]);
    acc[18] = fma(D48, mk, acc[18]);
    acc[19] = fma(D49, mk, acc[19]);
  }
  { const T mk = Mb[6];
    acc[0] = fma(D7, mk, acc[0]);
    acc[1] = fma(D13, mk, acc[1]);
    acc[2] = fma(D16, mk, acc[2]);
    acc[3] = fma(D17, mk, acc[3]);
    acc[4] = fma(D23, mk, acc[4]);
    acc[5] = fma(D26, mk, acc[5]);
    acc[6] = fma(D27, mk, acc[6]);
    acc[7] = fma(D30, mk, acc[7]);
    acc[8] = fma(D31, mk, acc[8]);
    acc[9] = fma(D32, mk, acc[9]);
    acc[10] = fma(D38, mk, acc[10]);
    acc[11] = fma(D41, mk, acc[11]);
    acc[12] = fma(D42, mk, acc[12]);
    acc[13] = fma(D45, mk, acc[13]);
    acc[14] = fma(D46, mk, acc[14]);
    acc[15] = fma(D47, mk, acc[15]);
    acc[16] = fma(D50, mk, acc[16]);
    acc[17] = fma(D51, mk, acc[17]);
    acc[18] = fma(D52, mk, acc[18]);
    acc[19] = fma(D53, mk, acc[19]);
  }
  { const T mk = Mb[7];
    acc[0] = fma(D8, mk, acc[0]);
    acc[1] = fma(D14, mk, acc[1]);
    acc[2] = fma(D17, mk, acc[2]);
    acc[3] = fma(D18, mk, acc[3]);
    acc[4] = fma(D24, mk, acc[4]);
    acc[5] = fma(D27, mk, acc[5]);
    acc[6] = fma(D28, mk, acc[6]);
    acc[7] = fma(D31, mk, acc[7]);
    acc[8] = fma(D32, mk, acc[8]);
    acc[9] = fma(D33, mk, acc[9]);
    acc[10] = fma(D39, mk, acc[10]);
    acc[11] = fma(D42, mk, acc[11]);
    acc[12] = fma(D43, mk, acc[12]);
    acc[13] = fma(D46, mk, acc[13]);
    acc[14] = fma(D47, mk, acc[14]);
    acc[15] = fma(D48, mk, acc[15]);
    acc[16] = fma(D51, mk, acc[16]);
    acc[17] = fma(D52, mk, acc[17]);
    acc[18] = fma(D53, mk, acc[18]);
    acc[19] = fma(D54, mk, acc[19]);
  }
  { const T mk = Mb[8];
    acc[0] = fma(D9, mk, acc[0]);
    acc[1] = fma(D15, mk, acc[1]);
    acc[2] = fma(D18, mk, acc[2]);
    acc[3] = fma(D19, mk, acc[3]);
    acc[4] = fma(D25, mk, acc[4]);
    acc[5] = fma(D28, mk, acc[5]);
    acc[6] = fma(D29, mk, acc[6]);
    acc[7] = fma(D32, mk, acc[7]);
    acc[8] = fma(D33, mk, acc[8]);
    acc[9] = fma(D34, mk, acc[9]);
    acc[10] = fma(D40, mk, acc[10]);
    acc[11] = fma(D43, mk, acc[11]);
    acc[12] = fma(D44, mk, acc[12]);
    acc[13] = fma(D47, mk, acc[13]);
    acc[14] = fma(D48, mk, acc[14]);
    acc[15] = fma(D49, mk, acc[15]);
    acc[16] = fma(D52, mk, acc[16]);
    acc[17] = fma(D53, mk, acc[17]);
    acc[18] = fma(D54, mk, acc[18]);
    acc[19] = fma(D55, mk, acc[19]);
  }
  { const T mk = Mb[9];
    acc[0] = fma(D10, mk, acc[0]);
    acc[1] = fma(D20, mk, acc[1]);
    acc[2] = fma(D21, mk, acc[2]);
    acc[3] = fma(D22, mk, acc[3]);
    acc[4] = fma(D35, mk, acc[4]);
    acc[5] = fma(D36, mk, acc[5]);
    acc[6] = fma(D37, mk, acc[6]);
    acc[7] = fma(D38, mk, acc[7]);
    acc[8] = fma(D39, mk, acc[8]);
    acc[9] = fma(D40, mk, acc[9]);
  }
  { const T mk = Mb[10];
    acc[0] = fma(D11, mk, acc[0]);
    acc[1] = fma(D21, mk, acc[1]);
    acc[2] = fma(D23, mk, acc[2]);
    acc[3] = fma(D24, mk, acc[3]);
    acc[4] = fma(D36, mk, acc[4]);
    acc[5] = fma(D38, mk, acc[5]);
    acc[6] = fma(D39, mk, acc[6]);
    acc[7] = fma(D41, mk, acc[7]);
    acc[8] = fma(D42, mk, acc[8]);
    acc[9] = fma(D43, mk, acc[9]);
  }
  { const T mk = Mb[11];
    acc[0] = fma(D12, mk, acc[0]);
    acc[1] = fma(D22, mk, acc[1]);
    acc[2] = fma(D24, mk, acc[2]);
    acc[3] = fma(D25, mk, acc[3]);
    acc[4] = fma(D37, mk, acc[4]);
    acc[5] = fma(D39, mk, acc[5]);
    acc[6] = fma(D40, mk, acc[6]);
    acc[7] = fma(D42, mk, acc[7]);
    acc[8] = fma(D43, mk, acc[8]);
    acc[9] = fma(D44, mk, acc[9]);
  }
  { const T mk = Mb[12];
    acc[0] = fma(D13, mk, acc[0]);
    acc[1] = fma(D23, mk, acc[1]);
    acc[2] = fma(D26, mk, acc[2]);
    acc[3] = fma(D27, mk, acc[3]);
    acc[4] = fma(D38, mk, acc[4]);
    acc[5] = fma(D41, mk, acc[5]);
    acc[6] = fma(D42, mk, acc[6]);
    acc[7] = fma(D45, mk, acc[7]);
    acc[8] = fma(D46, mk, acc[8]);
    acc[9] = fma(D47, mk, acc[9]);
  }
  { const T mk = Mb[13];
    acc[0] = fma(D14, mk, acc[0]);
    acc[1] = fma(D24, mk, acc[1]);
    acc[2] = fma(D27, mk, acc[2]);
    acc[3] = fma(D28, mk, acc[3]);
    acc[4] = fma(D39, mk, acc[4]);
    acc[5] = fma(D42, mk, acc[5]);
    acc[6] = fma(D43, mk, acc[6]);
    acc[7] = fma(D46, mk, acc[7]);
    acc[8] = fma(D47, mk, acc[8]);
    acc[9] = fma(D48, mk, acc[9]);
  }
  { const T mk = Mb[14];
    acc[0] = fma(D15, mk, acc[0]);
    acc[1] = fma(D25, mk, acc[1]);
    acc[2] = fma(D28, mk, acc[2]);
    acc[3] = fma(D29, mk, acc[3]);
    acc[4] = fma(D40, mk, acc[4]);
    acc[5] = fma(D43, mk, acc[5]);
    acc[6] = fma(D44, mk, acc[6]);
    acc[7] = fma(D47, mk, acc[7]);
    acc[8] = fma(D48, mk, acc[8]);
    acc[9] = fma(D49, mk, acc[9]);
  }
  { const T mk = Mb[15];
    acc[0] = fma(D16, mk, acc[0]);
    acc[1] = fma(D26, mk, acc[1]);
    acc[2] = fma(D30, mk, acc[2]);
    acc[3] = fma(D31, mk, acc[3]);
    acc[4] = fma(D41, mk, acc[4]);
    acc[5] = fma(D45, mk, acc[5]);
    acc[6] = fma(D46, mk, acc[6]);
    acc[7] = fma(D50, mk, acc[7]);
    acc[8] = fma(D51, mk, acc[8]);
    acc[9] = fma(D52, mk, acc[9]);
  }
  { const T mk = Mb[16];
    acc[0] = fma(D17, mk, acc[0]);
    acc[1] = fma(D27, mk, acc[1]);
    acc[2] = fma(D31, mk, acc[2]);
    acc[3] = fma(D32, mk, acc[3]);
    acc[4] = fma(D42, mk, acc[4]);
    acc[5] = fma(D46, mk, acc[5]);
    acc[6] = fma(D47, mk, acc[6]);
    acc[7] = fma(D51, mk, acc[7]);
    acc[8] = fma(D52, mk, acc[8]);
    acc[9] = fma(D53, mk, acc[9]);
  }
  { const T mk = Mb[17];
    acc[0] = fma(D18, mk, acc[0]);
    acc[1] = fma(D28, mk, acc[1]);
    acc[2] = fma(D32, mk, acc[2]);
    acc[3] = fma(D33, mk, acc[3]);
    acc[4] = fma(D43, mk, acc[4]);
    acc[5] = fma(D47, mk, acc[5]);
    acc[6] = fma(D48, mk, acc[6]);
    acc[7] = fma(D52, mk, acc[7]);
    acc[8] = fma(D53, mk, acc[8]);
    acc[9] = fma(D54, mk, acc[9]);
  }
  { const T mk = Mb[18];
    acc[0] = fma(D19, mk, acc[0]);
    acc[1] = fma(D29, mk, acc[1]);
    acc[2] = fma(D33, mk, acc[2]);
    acc[3] = fma(D34, mk, acc[3]);
    acc[4] = fma(D44, mk, acc[4]);
    acc[5] = fma(D48, mk, acc[5]);
    acc[6] = fma(D49, mk, acc[6]);
    acc[7] = fma(D53, mk, acc[7]);
    acc[8] = fma(D54, mk, acc[8]);
    acc[9] = fma(D55, mk, acc[9]);
  }
  { const T mk = Mb[19];
    acc[0] = fma(D20, mk, acc[0]);
    acc[1] = fma(D35, mk, acc[1]);
    acc[2] = fma(D36, mk, acc[2]);
    acc[3] = fma(D37, mk, acc[3]);
  }
  { const T mk = Mb[20];
    acc[0] = fma(D21, mk, acc[0]);
    acc[1] = fma(D36, mk, acc[1]);
    acc[2] = fma(D38, mk, acc[2]);
    acc[3] = fma(D39, mk, acc[3]);
  }
  { const T mk = Mb[21];
    acc[0] = fma(D22, mk, acc[0]);
    acc[1] = fma(D37, mk, acc[1]);
    acc[2] = fma(D39, mk, acc[2]);
    acc[3] = fma(D40, mk, acc[3]);
  }
  { const T mk = Mb[22];
    acc[0] = fma(D23, mk, acc[0]);
    acc[1] = fma(D38, mk, acc[1]);
    acc[2] = fma(D41, mk, acc[2]);
    acc[3] = fma(D42, mk, acc[3]);
  }
  { const T mk = Mb[23];
    acc[0] = fma(D24, mk, acc[0]);
    acc[1] = fma(D39, mk, acc[1]);
    acc[2] = fma(D42, mk, acc[2]);
    acc[3] = fma(D43, mk, acc[3]);
  }
  { const T mk = Mb[24];
    acc[0] = fma(D25, mk, acc[0]);
    acc[1] = fma(D40, mk, acc[1]);
    acc[2] = fma(D43, mk, acc[2]);
    acc[3] = fma(D44, mk, acc[3]);
  }
  { const T mk = Mb[25];
    acc[0] = fma(D26, mk, acc[0]);
    acc[1] = fma(D41, mk, acc[1]);
    acc[2] = fma(D45, mk, acc[2]);
    acc[3] = fma(D46, mk, acc[3]);
  }
  { const T mk = Mb[26];
    acc[0] = fma(D27, mk, acc[0]);
    acc[1] = fma(D42, mk, acc[1]);
    acc[2] = fma(D46, mk, acc[2]);
    acc[3] = fma(D47, mk, acc[3]);
  }
  { const T mk = Mb[27];
    acc[0] = fma(D28, mk, acc[0]);
    acc[1] = fma(D43, mk, acc[1]);
    acc[2] = fma(D47, mk, acc[2]);
    acc[3] = fma(D48, mk, acc[3]);
  }
  { const T mk = Mb[28];
    acc[0] = fma(D29, mk, acc[0]);
    acc[1] = fma(D44, mk, acc[1]);
    acc[2] = fma(D48, mk, acc[2]);
    acc[3] = fma(D49, mk, acc[3]);
  }
  { const T mk = Mb[29];
    acc[0] = fma(D30, mk, acc[0]);
    acc[1] = fma(D45, mk, acc[1]);
    acc[2] = fma(D50, mk, acc[2]);
    acc[3] = fma(D51, mk, acc[3]);
  }
  { const T mk = Mb[30];
    acc[0] = fma(D31, mk, acc[0]);
    acc[1] = fma(D46, mk, acc[1]);
    acc[2] = fma(D51, mk, acc[2]);
    acc[3] = fma(D52, mk, acc[3]);
  }
  { const T mk = Mb[31];
    acc[0] = fma(D32, mk, acc[0]);
    acc[1] = fma(D47, mk, acc[1]);
    acc[2] = fma(D52, mk, acc[2]);
    acc[3] = fma(D53, mk, acc[3]);
  }
  { const T mk = Mb[32];
    acc[0] = fma(D33, mk, acc[0]);
    acc[1] = fma(D48, mk, acc[1]);
    acc[2] = fma(D53, mk, acc[2]);
    acc[3] = fma(D54, mk, acc[3]);
  }
  { const T mk = Mb[33];
    acc[0] = fma(D34, mk, acc[0]);
    acc[1] = fma(D49, mk, acc[1]);
    acc[2] = fma(D54, mk, acc[2]);
    acc[3] = fma(D55, mk, acc[3]);
  }
  { const T mk = Mb[34];
    acc[0] = fma(D35, mk, acc[0]);
  }
  { const T mk = Mb[35];
    acc[0] = fma(D36, mk, acc[0]);
  }
  { const T mk = Mb[36];
    acc[0] = fma(D37, mk, acc[0]);
  }
  { const T mk = Mb[37];
    acc[0] = fma(D38, mk, acc[0]);
  }
  { const T mk = Mb[38];
    acc[0] = fma(D39, mk, acc[0]);
  }
  { const T mk = Mb[39];
    acc[0] = fma(D40, mk, acc[0]);
  }
  { const T mk = Mb[40];
    acc[0] = fma(D41, mk, acc[0]);
  }
  { const T mk = Mb[41];
    acc[0] = fma(D42, mk, acc[0]);
  }
  { const T mk = Mb[42];
    acc[0] = fma(D43, mk, acc[0]);
  }
  { const T mk = Mb[43];
    acc[0] = fma(D44, mk, acc[0]);
  }
  { const T mk = Mb[44];
    acc[0] = fma(D45, mk, acc[0]);
  }
  { const T mk = Mb[45];
    acc[0] = fma(D46, mk, acc[0]);
  }
  { const T mk = Mb[46];
    acc[0] = fma(D47, mk, acc[0]);
  }
  { const T mk = Mb[47];
    acc[0] = fma(D48, mk, acc[0]);
  }
  { const T mk = Mb[48];
    acc[0] = fma(D49, mk, acc[0]);
  }
  { const T mk = Mb[49];
    acc[0] = fma(D50, mk, acc[0]);
  }
  { const T mk = Mb[50];
    acc[0] = fma(D51, mk, acc[0]);
  }
  { const T mk = Mb[51];
    acc[0] = fma(D52, mk, acc[0]);
  }
  { const T mk = Mb[52];
    acc[0] = fma(D53, mk, acc[0]);
  }
  { const T mk = Mb[53];
    acc[0] = fma(D54, mk, acc[0]);
  }
  { const T mk = Mb[54];
    acc[0] = fma(D55, mk, acc[0]);
  }
}

// M2L, source order 1, expansion order 6: Msize 83, Lsize 56
template <typename T>
__device__ __forceinline__ void m2l_m1_p6(T x, T y, T z, const T* __restrict__ Mb, T* __restrict__ acc) {
  const T r2 = x * x + y * y + z * z;
  const T ir2 = T(1) / r2;
  const T D0 = rsqrt_t(r2);
  const T D1 = -(T(1) * (x * D0)) * ir2 * cinv<T>(1);
  const T D2 = -(T(1) * (y * D0)) * ir2 * cinv<T>(1);
  const T D3 = -(T(1) * (z * D0)) * ir2 * cinv<T>(1);
  const T D4 = -(T(3) * (T(2) * x * D1) + T(1) * (T(2) * D0)) * ir2 * cinv<T>(2);
  const T D5 = -(T(3) * (x * D2 + y * D1)) * ir2 * cinv<T>(2);
  const T D6 = -(T(3) * (x * D3 + z * D1)) * ir2 * cinv<T>(2);
  const T D7 = -(T(3) * (T(2) * y * D2) + T(1) * (T(2) * D0)) * ir2 * cinv<T>(2);
  const T D8 = -(T(3) * (y * D3 + z * D2)) * ir2 * cinv<T>(2);
  const T D9 = -(T(3) * (T(2) * z * D3) + T(1) * (T(2) * D0)) * ir2 * cinv<T>(2);
  const T D10 = -(T(5) * (T(3) * x * D4) + T(2) * (T(6) * D1)) * ir2 * cinv<T>(3);
  const T D11 = -(T(5) * (T(2) * x * D5 + y * D4) + T(2) * (T(2) * D2)) * ir2 * cinv<T>(3);
  const T D12 = -(T(5) * (T(2) * x * D6 + z * D4) + T(2) * (T(2) * D3)) * ir2 * cinv<T>(3);
  const T D13 = -(T(5) * (x * D7 + T(2) * y * D5) + T(2) * (T(2) * D1)) * ir2 * cinv<T>(3);
  const T D14 = -(T(5) * (x * D8 + y * D6 + z * D5)) * ir2 * cinv<T>(3);
  const T D15 = -(T(5) * (x * D9 + T(2) * z * D6) + T(2) * (T(2) * D1)) * ir2 * cinv<T>(3);
  const T D16 = -(T(5) * (T(3) * y * D7) + T(2) * (T(6) * D2)) * ir2 * cinv<T>(3);
  const T D17 = -(T(5) * (T(2) * y * D8 + z * D7) + T(2) * (T(2) * D3)) * ir2 * cinv<T>(3);
  const T D18 = -(T(5) * (y * D9 + T(2) * z * D8) + T(2) * (T(2) * D2)) * ir2 * cinv<T>(3);
  const T D19 = -(T(5) * (T(3) * z * D9) + T(2) * (T(6) * D3)) * ir2 * cinv<T>(3);
  const T D20 = -(T(7) * (T(4) * x * D10) + T(3) * (T(12) * D4)) * ir2 * cinv<T>(4);
  const T D21 = -(T(7) * (T(3) * x * D11 + y * D10) + T(3) * (T(6) * D5)) * ir2 * cinv<T>(4);
  const T D22 = -(T(7) * (T(3) * x * D12 + z * D10) + T(3) * (T(6) * D6)) * ir2 * cinv<T>(4);
  const T D23 = -(T(7) * (T(2) * x * D13 + T(2) * y * D11) + T(3) * (T(2) * D7 + T(2) * D4)) * ir2 * cinv<T>(4);
  const T D24 = -(T(7) * (T(2) * x * D14 + y * D12 + z * D11) + T(3) * (T(2) * D8)) * ir2 * cinv<T>(4);
  const T D25 = -(T(7) * (T(2) * x * D15 + T(2) * z * D12) + T(3) * (T(2) * D9 + T(2) * D4)) * ir2 * cinv<T>(4);
  const T D26 = -(T(7) * (x * D16 + T(3) * y * D13) + T(3) * (T(6) * D5)) * ir2 * cinv<T>(4);
  const T D27 = -(T(7) * (x * D17 + T(2) * y * D14 + z * D13) + T(3) * (T(2) * D6)) * ir2 * cinv<T>(4);
  const T D28 = -(T(7) * (x * D18 + y * D15 + T(2) * z * D14) + T(3) * (T(2) * D5)) * ir2 * cinv<T>(4);
  const T D29 = -(T(7) * (x * D19 + T(3) * z * D15) + T(3) * (T(6) * D6)) * ir2 * cinv<T>(4);
  const T D30 = -(T(7) * (T(4) * y * D16) + T(3) * (T(12) * D7)) * ir2 * cinv<T>(4);
  const T D31 = -(T(7) * (T(3) * y * D17 + z * D16) + T(3) * (T(6) * D8)) * ir2 * cinv<T>(4);
  const T D32 = -(T(7) * (T(2) * y * D18 + T(2) * z * D17) + T(3) * (T(2) * D9 + T(2) * D7)) * ir2 * cinv<T>(4);
  const T D33 = -(T(7) * (y * D19 + T(3) * z * D18) + T(3) * (T(6) * D8)) * ir2 * cinv<T>(4);
  const T D34 = -(T(7) * (T(4) * z * D19) + T(3) * (T(12) * D9)) * ir2 * cinv<T>(4);
  const T D35 = -(T(9) * (T(5) * x * D20) + T(4) * (T(20) * D10)) * ir2 * cinv<T>(5);
  const T D36 = -(T(9) * (T(4) * x * D21 + y * D20) + T(4) * (T(12) * D11)) * ir2 * cinv<T>(5);
  const T D37 = -(T(9) * (T(4) * x * D22 + z * D20) + T(4) * (T(12) * D12)) * ir2 * cinv<T>(5);
  const T D38 = -(T(9) * (T(3) * x * D23 + T(2) * y * D21) + T(4) * (T(6) * D13 + T(2) * D10)) * ir2 * cinv<T>(5);
  const T D39 = -(T(9) * (T(3) * x * D24 + y * D22 + z * D21) + T(4) * (T(6) * D14)) * ir2 * cinv<T>(5);
  const T D40 = -(T(9) * (T(3) * x * D25 + T(2) * z * D22) + T(4) * (T(6) * D15 + T(2) * D10)) * ir2 * cinv<T>(5);
  const T D41 = -(T(9) * (T(2) * x * D26 + T(3) * y * D23) + T(4) * (T(2) * D16 + T(6) * D11)) * ir2 * cinv<T>(5);
  const T D42 = -(T(9) * (T(2) * x * D27 + T(2) * y * D24 + z * D23) + T(4) * (T(2) * D17 + T(2) * D12)) * ir2 * cinv<T>(5);
  const T D43 = -(T(9) * (T(2) * x * D28 + y * D25 + T(2) * z * D24) + T(4) * (T(2) * D18 + T(2) * D11)) * ir2 * cinv<T>(5);
  const T D44 = -(T(9) * (T(2) * x * D29 + T(3) * z * D25) + T(4) * (T(2) * D19 + T(6) * D12)) * ir2 * cinv<T>(5);
  const T D45 = -(T(9) * (x * D30 + T(4) * y * D26) + T(4) * (T(12) * D13)) * ir2 * cinv<T>(5);
  const T D46 = -(T(9) * (x * D31 + T(3) * y * D27 + z * D26) + T(4) * (T(6) * D14)) * ir2 * cinv<T>(5);
  const T D47 = -(T(9) * (x * D32 + T(2) * y * D28 + T(2) * z * D27) + T(4) * (T(2) * D15 + T(2) * D13)) * ir2 * cinv<T>(5);
  const T D48 = -(T(9) * (x * D33 + y * D29 + T(3) * z * D28) + T(4) * (T(6) * D14)) * ir2 * cinv<T>(5);
  const T D49 = -(T(9) * (x * D34 + T(4) * z * D29) + T(4) * (T(12) * D15)) * ir2 * cinv<T>(5);
  const T D50 = -(T(9) * (T(5) * y * D30) + T(4) * (T(20) * D16)) * ir2 * cinv<T>(5);
  const T D51 = -(T(9) * (T(4) * y * D31 + z * D30) + T(4) * (T(12) * D17)) * ir2 * cinv<T>(5);
  const T D52 = -(T(9) * (T(3) * y * D32 + T(2) * z * D31) + T(4) * (T(6) * D18 + T(2) * D16)) * ir2 * cinv<T>(5);
  const T D53 = -(T(9) * (T(2) * y * D33 + T(3) * z * D32) + T(4) * (T(2) * D19 + T(6) * D17)) * ir2 * cinv<T>(5);
  const T D54 = -(T(9) * (y * D34 + T(4) * z * D33) + T(4) * (T(12) * D18)) * ir2 * cinv<T>(5);
  const T D55 = -(T(9) * (T(5) * z * D34) + T(4) * (T(20) * D19)) * ir2 * cinv<T>(5);
  const T D56 = -(T(11) * (T(6) * x * D35) + T(5) * (T(30) * D20)) * ir2 * cinv<T>(6);
  const T D57 = -(T(11) * (T(5) * x * D36 + y * D35) + T(5) * (T(20) * D21)) * ir2 * cinv<T>(6);
  const T D58 = -(T(11) * (T(5) * x * D37 + z * D35) + T(5) * (T(20) * D22)) * ir2 * cinv<T>(6);
  const T D59 = -(T(11) * (T(4) * x * D38 + T(2) * y * D36) + T(5) * (T(12) * D23 + T(2) * D20)) * ir2 * cinv<T>(6);
  const T D60 = -(T(11) * (T(4) * x * D39 + y * D37 + z * D36) + T(5) * (T(12) * D24)) * ir2 * cinv<T>(6);
  const T D61 = -(T(11) * (T(4) * x * D40 + T(2) * z * D37) + T(5) * (T(12) * D25 + T(2) * D20)) * ir2 * cinv<T>(6);
  const T D62 = -(T(11) * (T(3) * x * D41 + T(3) * y * D38) + T(5) * (T(6) * D26 + T(6) * D21)) * ir2 * cinv<T>(6);
  const T D63 = -(T(11) * (T(3) * x * D42 + T(2) * y * D39 + z * D38) + T(5) * (T(6) * D27 + T(2) * D22)) * ir2 * cinv<T>(6);
  const T D64 = -(T(11) * (T(3) * x * D43 + y * D40 + T(2) * z * D39) + T(5) * (T(6) * D28 + T(2) * D21)) * ir2 * cinv<T>(6);
  const T D65 = -(T(11) * (T(3) * x * D44 + T(3) * z * D40) + T(5) * (T(6) * D29 + T(6) * D22)) * ir2 * cinv<T>(6);
  const T D66 = -(T(11) * (T(2) * x * D45 + T(4) * y * D41) + T(5) * (T(2) * D30 + T(12) * D23)) * ir2 * cinv<T>(6);
  const T D67 = -(T(11) * (T(2) * x * D46 + T(3) * y * D42 + z * D41) + T(5) * (T(2) * D31 + T(6) * D24)) * ir2 * cinv<T>(6);
  const T D68 = -(T(11) * (T(2) * x * D47 + T(2) * y * D43 + T(2) * z * D42) + T(5) * (T(2) * D32 + T(2) * D25 + T(2) * D23)) * ir2 * cinv<T>(6);
  const T D69 = -(T(11) * (T(2) * x * D48 + y * D44 + T(3) * z * D43) + T(5) * (T(2) * D33 + T(6) * D24)) * ir2 * cinv<T>(6);
  const T D70 = -(T(11) * (T(2) * x * D49 + T(4) * z * D44) + T(5) * (T(2) * D34 + T(12) * D25)) * ir2 * cinv<T>(6);
  const T D71 = -(T(11) * (x * D50 + T(5) * y * D45) + T(5) * (T(20) * D26)) * ir2 * cinv<T>(6);
  const T D72 = -(T(11) * (x * D51 + T(4) * y * D46 + z * D45) + T(5) * (T(12) * D27)) * ir2 * cinv<T>(6);
  const T D73 = -(T(11) * (x * D52 + T(3) * y * D47 + T(2) * z * D46) + T(5) * (T(6) * D28 + T(2) * D26)) * ir2 * cinv<T>(6);
  const T D74 = -(T(11) * (x * D53 + T(2) * y * D48 + T(3) * z * D47) + T(5) * (T(2) * D29 + T(6) * D27)) * ir2 * cinv<T>(6);
  const T D75 = -(T(11) * (x * D54 + y * D49 + T(4) * z * D48) + T(5) * (T(12) * D28)) * ir2 * cinv<T>(6);
  const T D76 = -(T(11) * (x * D55 + T(5) * z * D49) + T(5) * (T(20) * D29)) * ir2 * cinv<T>(6);
  const T D77 = -(T(11) * (T(6) * y * D50) + T(5) * (T(30) * D30)) * ir2 * cinv<T>(6);
  const T D78 = -(T(11) * (T(5) * y * D51 + z * D50) + T(5) * (T(20) * D31)) * ir2 * cinv<T>(6);
  const T D79 = -(T(11) * (T(4) * y * D52 + T(2) * z * D51) + T(5) * (T(12) * D32 + T(2) * D30)) * ir2 * cinv<T>(6);
  const T D80 = -(T(11) * (T(3) * y * D53 + T(3) * z * D52) + T(5) * (T(6) * D33 + T(6) * D31)) * ir2 * cinv<T>(6);
  const T D81 = -(T(11) * (T(2) * y * D54 + T(4) * z * D53) + T(5) * (T(2) * D34 + T(12) * D32)) * ir2 * cinv<T>(6);
  const T D82 = -(T(11) * (y * D55 + T(5) * z * D54) + T(5) * (T(20) * D33)) * ir2 * cinv<T>(6);
  const T D83 = -(T(11) * (T(6) * z * D55) + T(5) * (T(30) * D34)) * ir2 * cinv<T>(6);
  { const T mk = Mb[0];
    acc[0] = fma(D1, mk, acc[0]);
    acc[1] = fma(D4, mk, acc[1]);
    acc[2] = fma(D5, mk, acc[2]);
    acc[3] = fma(D6, mk, acc[3]);
    acc[4] = fma(D10, mk, acc[4]);
    acc[5] = fma(D11, mk, acc[5]);
    acc[6] = fma(D12, mk, acc[6]);
    acc[7] = fma(D13, mk, acc[7]);
    acc[8] = fma(D14, mk, acc[8]);
    acc[9] = fma(D15, mk, acc[9]);
    acc[10] = fma(D20, mk, acc[10]);
    acc[11] = fma(D21, mk, acc[11]);
    acc[12] = fma(D22, mk, acc[12]);
    acc[13] = fma(D23, mk, acc[13]);
    acc[14] = fma(D24, mk, acc[14]);
    acc[15] = fma(D25, mk, acc[15]);
    acc[16] = fma(D26, mk, acc[16]);
    acc[17] = fma(D27, mk, acc[17]);
    acc[18] = fma(D28, mk, acc[18]);
    acc[19] = fma(D29, mk, acc[19]);
    acc[20] = fma(D35, mk, acc[20]);
    acc[21] = fma(D36, mk, acc[21]);
    acc[22] = fma(D37, mk, acc[22]);
    acc[23] = fma(D38, mk, acc[23]);
    acc[24] = fma(D39, mk, acc[24]);
    acc[25] = fma(D40, mk, acc[25]);
    acc[26] = fma(D41, mk, acc[26]);
    acc[27] = fma(D42, mk, acc[27]);
    acc[28] = fma(D43, mk, acc[28]);
    acc[29] = fma(D44, mk, acc[29]);
    acc[30] = fma(D45, mk, acc[30]);
    acc[31] = fma(D46, mk, acc[31]);
    acc[32] = fma(D47, mk, acc[32]);
    acc[33] = fma(D48, mk, acc[33]);
    acc[34] = fma(D49, mk, acc[34]);
    acc[35] = fma(D56, mk, acc[35]);
    acc[36] = fma(D57, mk, acc[36]);
    acc[37] = fma(D58, mk, acc[37]);
    acc[38] = fma(D59, mk, acc[38]);
    acc[39] = fma(D60, mk, acc[39]);
    acc[40] = fma(D61, mk, acc[40]);
    acc[41] = fma(D62, mk, acc[41]);
    acc[42] = fma(D63, mk, acc[42]);
    acc[43] = fma(D64, mk, acc[43]);
    acc[44] = fma(D65, mk, acc[44]);
    acc[45] = fma(D66, mk, acc[45]);
    acc[46] = fma(D67, mk, acc[46]);
    acc[47] = fma(D68, mk, acc[47]);
    acc[48] = fma(D69, mk, acc[48]);
    acc[49] = fma(D70, mk, acc[49]);
    acc[50] = fma(D71, mk, acc[50]);
    acc[51] = fma(D72, mk, acc[51]);
    acc[52] = fma(D73, mk, acc[52]);
    acc[53] = fma(D74, mk, acc[53]);
    acc[54] = fma(D75, mk, acc[54]);
    acc[55] = fma(D76, mk, acc[55]);
  }
  { const T mk = Mb[1];
    acc[0] = fma(D2, mk, acc[0]);
    acc[1] = fma(D5, mk, acc[1]);
    acc[2] = fma(D7, mk, acc[2]);
    acc[3] = fma(D8, mk, acc[3]);
    acc[4] = fma(D11, mk, acc[4]);
    acc[5] = fma(D13, mk, acc[5]);
    acc[6] = fma(D14, mk, acc[6]);
    acc[7] = fma(D16, mk, acc[7]);
    acc[8] = fma(D17, mk, acc[8]);
    acc[9] = fma(D18, mk, acc[9]);
    acc[10] = fma(D21, mk, acc[10]);
    acc[11] = fma(D23, mk, acc[11]);
    acc[12] = fma(D24, mk, acc[12]);
    acc[13] = fma(D26, mk, acc[13]);
    acc[14] = fma(D27, mk, acc[14]);
    acc[15] = fma(D28, mk, acc[15]);
    acc[16] = fma(D30, mk, acc[16]);
    acc[17] = fma(D31, mk, acc[17]);
    acc[18] = fma(D32, mk, acc[18]);
    acc[19] = fma(D33, mk, acc[19]);
    acc[20] = fma(D36, mk, acc[20]);
    acc[21] = fma(D38, mk, acc[21]);
    acc[22] = fma(D39, mk, acc[22]);
    acc[23] = fma(D41, mk, acc[23]);
    acc[24] = fma(D42, mk, acc[24]);
    acc[25] = fma(D43, mk, acc[25]);
    acc[26] = fma(D45, mk, acc[26]);
    acc[27] = fma(D46, mk, acc[27]);
    acc[28] = fma(D47, mk, acc[28]);
    acc[29] = fma(D48, mk, acc[29]);
    acc[30] = fma(D50, mk, acc[30]);
    acc[31] = fma(D51, mk, acc[31]);
    acc[32] = fma(D52, mk, acc[32]);
    acc[33] = fma(D53, mk, acc[33]);
    acc[34] = fma(D54, mk, acc[34]);
    acc[35] = fma(D57, mk, acc[35]);
    acc[36] = fma(D59, mk, acc[36]);
    acc[37] = fma(D60, mk, acc[37]);
    acc[38] = fma(D62, mk, acc[38]);
    acc[39] = fma(D63, mk, acc[39]);
    acc[40] = fma(D64, mk, acc[40]);
    acc[41] = fma(D66, mk, acc[41]);
    acc[42] = fma(D67, mk, acc[42]);
    acc[43] = fma(D68, mk, acc[43]);
    acc[44] = fma(D69, mk, acc[44]);
    acc[45] = fma(D71, mk, acc[45]);
    acc[46] = fma(D72, mk, acc[46]);
    acc[47] = fma(D73, mk, acc[47]);
    acc[48] = fma(D74, mk, acc[48]);
    acc[49] = fma(D75, mk, acc[49]);
    acc[50] = fma(D77, mk, acc[50]);
    acc[51] = fma(D78, mk, acc[51]);
    acc[52] = fma(D79, mk, acc[52]);
    acc[53] = fma(D80, mk, acc[53]);
    acc[54] = fma(D81, mk, acc[54]);
    acc[55] = fma(D82, mk, acc[55]);
  }
  { const T mk = Mb[2];
    acc[0] = fma(D3, mk, acc[0]);
    acc[1] = fma(D6, mk, acc[1]);
    acc[2] = fma(D8, mk, acc[2]);
    acc[3] = fma(D9, mk, acc[3]);
    acc[4] = fma(D12, mk, acc[4]);
    acc[5] = fma(D14, mk, acc[5]);
    acc[6] = fma(D15, mk, acc[6]);
    acc[7] = fma(D17, mk, acc[7]);
    acc[8] = fma(D18, mk, acc[8]);
    acc[9] = fma(D19, mk, acc[9]);
    acc[10] = fma(D22, mk, acc[10]);
    acc[11] = fma(D24, mk, acc[11]);
    acc[12] = fma(D25, mk, acc[12]);
    acc[13] = fma(D27, mk, acc[13]);
    acc[14] = fma(D28, mk, acc[14]);
    acc[15] = fma(D29, mk, acc[15]);
    acc[16] = fma(D31, mk, acc[16]);
    acc[17] = fma(D32, mk, acc[17]);
    acc[18] = fma(D33, mk, acc[18]);
    acc[19] = fma(D34, mk, acc[19]);
    acc[20] = fma(D37, mk, acc[20]);
    acc[21] = fma(D39, mk, acc[21]);
    acc[22] = fma(D40, mk, acc[22]);
    acc[23] = fma(D42, mk, acc[23]);
    acc[24] = fma(D43, mk, acc[24]);
    acc[25] = fma(D44, mk, acc[25]);
    acc[26] = fma(D46, mk, acc[26]);
    acc[27] = fma(D47, mk, acc[27]);
    acc[28] = fma(D48, mk, acc[28]);
    acc[29] = fma(D49, mk, acc[29]);
    acc[30] = fma(D51, mk, acc[30]);
    acc[31] = fma(D52, mk, acc[31]);
    acc[32] = fma(D53, mk, acc[32]);
    acc[33] = fma(D54, mk, acc[33]);
    acc[34] = fma(D55, mk, acc[34]);
    acc[35] = fma(D58, mk, acc[35]);
    acc[36] = fma(D60, mk, acc[36]);
    acc[37] = fma(D61, mk, acc[37]);
    acc[38] = fma(D63, mk, acc[38]);
    acc[39] = fma(D64, mk, acc[39]);
    acc[40] = fma(D65, mk, acc[40]);
    acc[41] = fma(D67, mk, acc[41]);
    acc[42] = fma(D68, mk, acc[42]);
    acc[43] = fma(D69, mk, acc[43]);
    acc[44] = fma(D70, mk, acc[44]);
    acc[45] = fma(D72, mk, acc[45]);
    acc[46] = fma(D73, mk, acc[46]);
    acc[47] = fma(D74, mk, acc[47]);
    acc[48] = fma(D75, mk, acc[48]);
    acc[49] = fma(D76, mk, acc[49]);
    acc[50] = fma(D78, mk, acc[50]);
    acc[51] = fma(D79, mk, acc[51]);
    acc[52] = fma(D80, mk, acc[52]);
    acc[53] = fma(D81, mk, acc[53]);
    acc[54] = fma(D82, mk, acc[54]);
    acc[55] = fma(D83, mk, acc[55]);
  }
  { const T mk = Mb[3];
    acc[0] = fma(D4, mk, acc[0]);
    acc[1] = fma(D10, mk, acc[1]);
    acc[2] = fma(D11, mk, acc[2]);
    acc[3] = fma(D12, mk, acc[3]);
    acc[4] = fma(D20, mk, acc[4]);
    acc[5] = fma(D21, mk, acc[5]);
    acc[6] = fma(D22, mk, acc[6]);
    acc[7] = fma(D23, mk, acc[7]);
    acc[8] = fma(D24, mk, acc[8]);
    acc[9] = fma(D25, mk, acc[9]);
    acc[10] = fma(D35, mk, acc[10]);
    acc[11] = fma(D36, mk, acc[11]);
    acc[12] = fma(D37, mk, acc[12]);
    acc[13] = fma(D38, mk, acc[13]);
    acc[14] = fma(D39, mk, acc[14]);
    acc[15] = fma(D40, mk, acc[15]);
    acc[16] = fma(D41, mk, acc[16]);
    acc[17] = fma(D42, mk, acc[17]);
    acc[18] = fma(D43, mk, acc[18]);
    acc[19] = fma(D44, mk, acc[19]);
    acc[20] = fma(D56, mk, acc[20]);
    acc[21] = fma(D57, mk, acc[21]);
    acc[22] = fma(D58, mk, acc[22]);
    acc[23] = fma(D59, mk, acc[23]);
    acc[24] = fma(D60, mk, acc[24]);
    acc[25] = fma(D61, mk, acc[25]);
    acc[26] = fma(D62, mk, acc[26]);
    acc[27] = fma(D63, mk, acc[27]);
    acc[28] = fma(D64, mk, acc[28]);
    acc[29] = fma(D65, mk, acc[29]);
    acc[30] = fma(D66, mk, acc[30]);
    acc[31] = fma(D67, mk, acc[31]);
    acc[32] = fma(D68, mk, acc[32]);
    acc[33] = fma(D69, mk, acc[33]);
    acc[34] = fma(D70, mk, acc[34]);
  }
  { const T mk = Mb[4];
    acc[0] = fma(D5, mk, acc[0]);
    acc[1] = fma(D11, mk, acc[1]);
    acc[2] = fma(D13, mk, acc[2]);
    acc[3] = fma(D14, mk, acc[3]);
    acc[4] = fma(D21, mk, acc[4]);
    acc[5] = fma(D23, mk, acc[5]);
    acc[6] = fma(D24, mk, acc[6]);
    acc[7] = fma(D26, mk, acc[7]);
    acc[8] = fma(D27, mk, acc[8]);
    acc[9] = fma(D28, mk, acc[9]);
    acc[10] = fma(D36, mk, acc[10]);
    acc[11] = fma(D38, mk, acc[11]);
    acc[12] = fma(D39, mk, acc[12]);
    acc[13] = fma(D41, mk, acc[13]);
    acc[14] = fma(D42, mk, acc[14]);
    acc[15] = fma(D43, mk, acc[15]);
    acc[16] = fma(D45, mk, acc[16]);
    acc[17] = fma(D46, mk, acc[17]);
    acc[18] = fma(D47, mk, acc[18]);
    acc[19] = fma(D48, mk, acc[19]);
    acc[20] = fma(D57, mk, acc[20]);
    acc[21] = fma(D59, mk, acc[21]);
    acc[22] = fma(D60, mk, acc[22]);
    acc[23] = fma(D62, mk, acc[23]);
    acc[24] = fma(D63, mk, acc[24]);
    acc[25] = fma(D64, mk, acc[25]);
    acc[26] = fma(D66, mk, acc[26]);
    acc[27] = fma(D67, mk, acc[27]);
    acc[28] = fma(D68, mk, acc[28]);
    acc[29] = fma(D69, mk, acc[29]);
    acc[30] = fma(D71, mk, acc[30]);
    acc[31] = fma(D72, mk, acc[31]);
    acc[32] = fma(D73, mk, acc[32]);
    acc[33] = fma(D74, mk, acc[33]);
    acc[34] = fma(D75, mk, acc[34]);
  }
  { const T mk = Mb[5];
    acc[0] = fma(D6, mk, acc[0]);
    acc[1] = fma(D12, mk, acc[1]);
    acc[2] = fma(D14, mk, acc[2]);
    acc[3] = fma(D15, mk, acc[3]);
    acc[4] = fma(D22, mk, acc[4]);
    acc[5] = fma(D24, mk, acc[5]);
    acc[6] = fma(D25, mk, acc[6]);
    acc[7] = fma(D27, mk, acc[7]);
    acc[8] = fma(D28, mk, acc[8]);
    acc[9] = fma(D29, mk, acc[9]);
    acc[10] = fma(D37, mk, acc[10]);
    acc[11] = fma(D39, mk, acc[11]);
    acc[12] = fma(D40, mk, acc[12]);
    acc[13] = fma(D42, mk, acc[13]);
    acc[14] = fma(D43, mk, acc[14]);
    acc[15] = fma(D44, mk, acc[15]);
    acc[16] = fma(D46, mk, acc[16]);
    acc[17] = fma(D47, mk, acc[17]);
    acc[18] = fma(D48, mk, acc[18]);
    acc[19] = fma(D49, mk, acc[19]);
    acc[20] = fma(D58, mk, acc[20]);
    acc[21] = fma(D60, mk, acc[21]);
    acc[22] = fma(D61, mk, acc[22]);
    acc[23] = fma(D63, mk, acc[23]);
    acc[24] = fma(D64, mk, acc[24]);
    acc[25] = fma(D65, mk, acc[25]);
    acc[26] = fma(D67, mk, acc[26]);
    acc[27] = fma(D68, mk, acc[27]);
    acc[28] = fma(D69, mk, acc[28]);
    acc[29] = fma(D70, mk, acc[29]);
    acc[30] = fma(D72, mk, acc[30]);
    acc[31] = fma(D73, mk, acc[31]);
    acc[32] = fma(D74, mk, acc[32]);
    acc[33] = fma(D75, mk, acc[33]);
    acc[34] = fma(D76, mk, acc[34]);
  }
  { const T mk = Mb[6];
    acc[0] = fma(D7, mk, acc[0]);
    acc[1] = fma(D13, mk, acc[1]);
    acc[2] = fma(D16, mk, acc[2]);
    acc[3] = fma(D17, mk, acc[3]);
    acc[4] = fma(D23, mk, acc[4]);
    acc[5] = fma(D26, mk, acc[5]);
    acc[6] = fma(D27, mk, acc[6]);
    acc[7] = fma(D30, mk, acc[7]);
    acc[8] = fma(D31, mk, acc[8]);
    acc[9] = fma(D32, mk, acc[9]);
    acc[10] = fma(D38, mk, acc[10]);
    acc[11] = fma(D41, mk, acc[11]);
    acc[12] = fma(D42, mk, acc[12]);
    acc[13] = fma(D45, mk, acc[13]);
    acc[14] = fma(D46, mk, acc[14]);
    acc[15] = fma(D47, mk, acc[15]);
    acc[16] = fma(D50, mk, acc[16]);
    acc[17] = fma(D51, mk, acc[17]);
    acc[18] = fma(D52, mk, acc[18]);
    acc[19] = fma(D53, mk, acc[19]);
    acc[20] = fma(D59, mk, acc[20]);
    acc[21] = fma(D62, mk, acc[21]);
    acc[22] = fma(D63, mk, acc[22]);
    acc[23] = fma(D66, mk, acc[23]);
    acc[24] = fma(D67, mk, acc[24]);
    acc[25] = fma(D68, mk, acc[25]);
    acc[26] = fma(D71, mk, acc[26]);
    acc[27] = fma(D72, mk, acc[27]);
    acc[28] = fma(D73, mk, acc[28]);
    acc[29] = fma(D74, mk, acc[29]);
    acc[30] = fma(D77, mk, acc[30]);
    acc[31] = fma(D78, mk, acc[31]);
    acc[32] = fma(D79, mk, acc[32]);
    acc[33] = fma(D80, mk, acc[33]);
    acc[34] = fma(D81, mk, acc[34]);
  }
  { const T mk = Mb[7];
    acc[0] = fma(D8, mk, acc[0]);
    acc[1] = fma(D14, mk, acc[1]);
    acc[2] = fma(D17, mk, acc[2]);
    acc[3] = fma(D18, mk, acc[3]);
    acc[4] = fma(D24, mk, acc[4]);
    acc[5] = fma(D27, mk, acc[5]);
    acc[6] = fma(D28, mk, acc[6]);
    acc[7] = fma(D31, mk, acc[7]);
    acc[8] = fma(D32, mk, acc[8]);
    acc[9] = fma(D33, mk, acc[9]);
    acc[10] = fma(D39, mk, acc[10]);
    acc[11] = fma(D42, mk, acc[11]);
    acc[12] = fma(D43, mk, acc[12]);
    acc[13] = fma(D46, mk, acc[13]);
    acc[14] = fma(D47, mk, acc[14]);
    acc[15] = fma(D48, mk, acc[15]);
    acc[16] = fma(D51, mk, acc[16]);
    acc[17] = fma(D52, mk, acc[17]);
    acc[18] = fma(D53, mk, acc[18]);
    acc[19] = fma(D54, mk, acc[19]);
    acc[20] = fma(D60, mk, acc[20]);
    acc[21] = fma(D63, mk, acc[21]);
    acc[22] = fma(D64, mk, acc[22]);
    acc[23] = fma(D67, mk, acc[23]);
    acc[24] = fma(D68, mk, acc[24]);
    acc[25] = fma(D69, mk, acc[25]);
    acc[26] = fma(D72, mk, acc[26]);
    acc[27] = fma(D73, mk, acc[27]);
    acc[28] = fma(D74, mk, acc[28]);
    acc[29] = fma(D75, mk, acc[29]);
    acc[30] = fma(D78, mk, acc[30]);
    acc[31] = fma(D79, mk, acc[31]);
    acc[32] = fma(D80, mk, acc[32]);
    acc[33] = fma(D81, mk, acc[33]);
    acc[34] = fma(D82, mk, acc[34]);
  }
  { const T mk = Mb[8];
    acc[0] = fma(D9, mk, acc[0]);
    acc[1] = fma(D15, mk, acc[1]);
    acc[2] = fma(D18, mk, acc[2]);
    acc[3] = fma(D19, mk, acc[3]);
    acc[4] = fma(D25, mk, acc[4]);
    acc[5] = fma(D28, mk, acc[5]);
    acc[6] = fma(D29, mk, acc[6]);
    acc[7] = fma(D32, mk, acc[7]);
    acc[8] = fma(D33, mk, acc[8]);
    acc[9] = fma(D34, mk, acc[9]);
    acc[10] = fma(D40, mk, acc[10]);
    acc[11] = fma(D43, mk, acc[11]);
    acc[12] = fma(D44, mk, acc[12]);
    acc[13] = fma(D47, mk, acc[13]);
    acc[14] = fma(D48, mk, acc[14]);
    acc[15] = fma(D49, mk, acc[15]);
    acc[16] = fma(D52, mk, acc[16]);
    acc[17] = fma(D53, mk, acc[17]);
    acc[18] = fma(D54, mk, acc[18]);
    acc[19] = fma(D55, mk, acc[19]);
    acc[20] = fma(D61, mk, acc[20]);
    acc[21] = fma(D64, mk, acc[21]);
    acc[22] = fma(D65, mk, acc[22]);
    acc[23] = fma(D68, mk, acc[23]);
    acc[24] = fma(D69, mk, acc[24]);
    acc[25] = fma(D70, mk, acc[25]);
    acc[26] = fma(D73, mk, acc[26]);
    acc[27] = fma(D74, mk, acc[27]);
    acc[28] = fma(D75, mk, acc[28]);
    acc[29] = fma(D76, mk, acc[29]);
    acc[30] = fma(D79, mk, acc[30]);
    acc[31] = fma(D80, mk, acc[31]);
    acc[32] = fma(D81, mk, acc[32]);
    acc[33] = fma(D82, mk, acc[33]);
    acc[34] = fma(D83, mk, acc[34]);
  }
  { const T mk = Mb[9];
    acc[0] = fma(D10, mk, acc[0]);
    acc[1] = fma(D20, mk, acc[1]);
    acc[2] = fma(D21, mk, acc[2]);
    acc[3] = fma(D22, mk, acc[3]);
    acc[4] = fma(D35, mk, acc[4]);
    acc[5] = fma(D36, mk, acc[5]);
    acc[6] = fma(D37, mk, acc[6]);
    acc[7] = fma(D38, mk, acc[7]);
    acc[8] = fma(D39, mk, acc[8]);
    acc[9] = fma(D40, mk, acc[9]);
    acc[10] = fma(D56, mk, acc[10]);
    acc[11] = fma(D57, mk, acc[11]);
    acc[12] = fma(D58, mk, acc[12]);
    acc[13] = fma(D59, mk, acc[13]);
    acc[14] = fma(D60, mk, acc[14]);
    acc[15] = fma(D61, mk, acc[15]);
    acc[16] = fma(D62, mk, acc[16]);
    acc[17] = fma(D63, mk, acc[17]);
    acc[18] = fma(D64, mk, acc[18]);
    acc[19] = fma(D65, mk, acc[19]);
  }
  { const T mk = Mb[10];
    acc[0] = fma(D11, mk, acc[0]);
    acc[1] = fma(D21, mk, acc[1]);
    acc[2] = fma(D23, mk, acc[2]);
    acc[3] = fma(D24, mk, acc[3]);
    acc[4] = fma(D36, mk, acc[4]);
    acc[5] = fma(D38, mk, acc[5]);
    acc[6] = fma(D39, mk, acc[6]);
    acc[7] = fma(D41, mk, acc[7]);
    acc[8] = fma(D42, mk, acc[8]);
    acc[9] = fma(D43, mk, acc[9]);
    acc[10] = fma(D57, mk, acc[10]);
    acc[11] = fma(D59, mk, acc[11]);
    acc[12] = fma(D60, mk, acc[12]);
    acc[13] = fma(D62, mk, acc[13]);
    acc[14] = fma(D63, mk, acc[14]);
    acc[15] = fma(D64, mk, acc[15]);
    acc[16] = fma(D66, mk, acc[16]);
    acc[17] = fma(D67, mk, acc[17]);
    acc[18] = fma(D68, mk, acc[18]);
    acc[19] = fma(D69, mk, acc[19]);
  }
  { const T mk = Mb[11];
    acc[0] = fma(D12, mk, acc[0]);
    acc[1] = fma(D22, mk, acc[1]);
    acc[2] = fma(D24, mk, acc[2]);
    acc[3] = fma(D25, mk, acc[3]);
    acc[4] = fma(D37, mk, acc[4]);
    acc[5] = fma(D39, mk, acc[5]);
    acc[6] = fma(D40, mk, acc[6]);
    acc[7] = fma(D42, mk, acc[7]);
    acc[8] = fma(D43, mk, acc[8]);
    acc[9] = fma(D44, mk, acc[9]);
    acc[10] = fma(D58, mk, acc[10]);
    acc[11] = fma(D60, mk, acc[11]);
    acc[12] = fma(D61, mk, acc[12]);
    acc[13] = fma(D63, mk, acc[13]);
    acc[14] = fma(D64, mk, acc[14]);
    acc[15] = fma(D65, mk, acc[15]);
    acc[16] = fma(D67, mk, acc[16]);
    acc[17] = fma(D68, mk, acc[17]);
    acc[18] = fma(D69, mk, acc[18]);
    acc[19] = fma(D70, mk, acc[19]);
  }
  { const T mk = Mb[12];
    acc[0] = fma(D13, mk, acc[0]);
    acc[1] = fma(D23, mk, acc[1]);
    acc[2] = fma(D26, mk, acc[2]);
    acc[3] = fma(D27, mk, acc[3]);
    acc[4] = fma(D38, mk, acc[4]);
    acc[5] = fma(D41, mk, acc[5]);
    acc[6] = fma(D42, mk, acc[6]);
    acc[7] = fma(D45, mk, acc[7]);
    acc[8] = fma(D46, mk, acc[8]);
    acc[9] = fma(D47, mk, acc[9]);
    acc[10] = fma(D59, mk, acc[10]);
    acc[11] = fma(D62, mk, acc[11]);
    acc[12] = fma(D63, mk, acc[12]);
    acc[13] = fma(D66, mk, acc[13]);
    acc[14] = fma(D67, mk, acc[14]);
    acc[15] = fma(D68, mk, acc[15]);
    acc[16] = fma(D71, mk, acc[16]);
    acc[17] = fma(D72, mk, acc[17]);
    acc[18] = fma(D73, mk, acc[18]);
    acc[19] = fma(D74, mk, acc[19]);
  }
  { const T mk = Mb[13];
    acc[0] = fma(D14, mk, acc[0]);
    acc[1] = fma(D24, mk, acc[1]);
    acc[2] = fma(D27, mk, acc[2]);
    acc[3] = fma(D28, mk, acc[3]);
    acc[4] = fma(D39, mk, acc[4]);
    acc[5] = fma(D42, mk, acc[5]);
    acc[6] = fma(D43, mk, acc[6]);
    acc[7] = fma(D46, mk, acc[7]);
    acc[8] = fma(D47, mk, acc[8]);
    acc[9] = fma(D48, mk, acc[9]);
    acc[10] = fma(D60, mk, acc[10]);
    acc[11] = fma(D63, mk, acc[11]);
    acc[12] = fma(D64, mk, acc[12]);
    acc[13] = fma(D67, mk, acc[13]);
    acc[14] = fma(D68, mk, acc[14]);
    acc[15] = fma(D69, mk, acc[15]);
    acc[16] = fma(D72, mk, acc[16]);
    acc[17] = fma(D73, mk, acc[17]);
    acc[18] = fma(D74, mk, acc[18]);
    acc[19] = fma(D75, mk, acc[19]);
  }
  { const T mk = Mb[14];
    acc[0] = fma(D15, mk, acc[0]);
    acc[1] = fma(D25, mk, acc[1]);
    acc[2] = fma(D28, mk, acc[2]);
    acc[3] = fma(D29, mk, acc[3]);
    acc[4] = fma(D40, mk, acc[4]);
    acc[5] = fma(D43, mk, acc[5]);
    acc[6] = fma(D44, mk, acc[6]);
    acc[7] = fma(D47, mk, acc[7]);
    acc[8] = fma(D48, mk, acc[8]);
    acc[9] = fma(D49, mk, acc[9]);
    acc[10] = fma(D61, mk, acc[10]);
    acc[11] = fma(D64, mk, acc[11]);
    acc[12] = fma(D65, mk, acc[12]);
    acc[13] = fma(D68, mk, acc[13]);
    acc[14] = fma(D69, mk, acc[14]);
    acc[15] = fma(D70, mk, acc[15]);
    acc[16] = fma(D73, mk, acc[16]);
    acc[17] = fma(D74, mk, acc[17]);
    acc[18] = fma(D75, mk, acc[18]);
    acc[19] = fma(D76, mk, acc[19]);
  }
  { const T mk = Mb[15];
    acc[0] = fma(D16, mk, acc[0]);
    acc[1] = fma(D26, mk, acc[1]);
    acc[2] = fma(D30, mk, acc[2]);
    acc[3] = fma(D31, mk, acc[3]);
    acc[4] = fma(D41, mk, acc[4]);
    acc[5] = fma(D45, mk, acc[5]);
    acc[6] = fma(D46, mk, acc[6]);
    acc[7] = fma(D50, mk, acc[7]);
    acc[8] = fma(D51, mk, acc[8]);
    acc[9] = fma(D52, mk, acc[9]);
    acc[10] = fma(D62, mk, acc[10]);
    acc[11] = fma(D66, mk, acc[11]);
    acc[12] = fma(D67, mk, acc[12]);
    acc[13] = fma(D71, mk, acc[13]);
    acc[14] = fma(D72, mk, acc[14]);
    acc[15] = fma(D73, mk, acc[15]);
    acc[16] = fma(D77, mk, acc[16]);
    acc[17] = fma(D78, mk, acc[17]);
    acc[18] = fma(D79, mk, acc[18]);
    acc[19] = fma(D80, mk, acc[19]);
  }
  { const T mk = Mb[16];
    acc[0] = fma(D17, mk, acc[0]);
    acc[1] = fma(D27, mk, acc[1]);
    acc[2] = fma(D31, mk, acc[2]);
    acc[3] = fma(D32, mk, acc[3]);
    acc[4] = fma(D42, mk, acc[4]);
    acc[5] = fma(D46, mk, acc[5]);
    acc[6] = fma(D47, mk, acc[6]);
    acc[7] = fma(D51, mk, acc[7]);
    acc[8] = fma(D52, mk, acc[8]);
    acc[9] = fma(D53, mk, acc[9]);
    acc[10] = fma(D63, mk, acc[10]);
    acc[11] = fma(D67, mk, acc[11]);
    acc[12] = fma(D68, mk, acc[12]);
    acc[13] = fma(D72, mk, acc[13]);
    acc[14] = fma(D73, mk, acc[14]);
    acc[15] = fma(D74, mk, acc[15]);
    acc[16] = fma(D78, mk, acc[16]);
    acc[17] = fma(D79, mk, acc[17]);
    acc[18] = fma(D80, mk, acc[18]);
    acc[19] = fma(D81, mk, acc[19]);
  }
  { const T mk = Mb[17];
    acc[0] = fma(D18, mk, acc[0]);
    acc[1] = fma(D28, mk, acc[1]);
    acc[2] = fma(D32, mk, acc[2]);
    acc[3] = fma(D33, mk, acc[3]);
    acc[4] = fma(D43, mk, acc[4]);
    acc[5] = fma(D47, mk, acc[5]);
    acc[6] = fma(D48, mk, acc[6]);
    acc[7] = fma(D52, mk, acc[7]);
    acc[8] = fma(D53, mk, acc[8]);
    acc[9] = fma(D54, mk, acc[9]);
    acc[10] = fma(D64, mk, acc[10]);
    acc[11] = fma(D68, mk, acc[11]);
    acc[12] = fma(D69, mk, acc[12]);
    acc[13] = fma(D73, mk, acc[13]);
    acc[14] = fma(D74, mk, acc[14]);
    acc[15] = fma(D75, mk, acc[15]);
    acc[16] = fma(D79, mk, acc[16]);
    acc[17] = fma(D80, mk, acc[17]);
    acc[18] = fma(D81, mk, acc[18]);
    acc[19] = fma(D82, mk, acc[19]);
  }
  { const T mk = Mb[18];
    acc[0] = fma(D19, mk, acc[0]);
    acc[1] = fma(D29, mk, acc[1]);
    acc[2] = fma(D33, mk, acc[2]);
    acc[3] = fma(D34, mk, acc[3]);
    acc[4] = fma(D44, mk, acc[4]);
    acc[5] = fma(D48, mk, acc[5]);
    acc[6] = fma(D49, mk, acc[6]);
    acc[7] = fma(D53, mk, acc[7]);
    acc[8] = fma(D54, mk, acc[8]);
    acc[9] = fma(D55, mk, acc[9]);
    acc[10] = fma(D65, mk, acc[10]);
    acc[11] = fma(D69, mk, acc[11]);
    acc[12] = fma(D70, mk, acc[12]);
    acc[13] = fma(D74, mk, acc[13]);
    acc[14] = fma(D75, mk, acc[14]);
    acc[15] = fma(D76, mk, acc[15]);
    acc[16] = fma(D80, mk, acc[16]);
    acc[17] = fma(D81, mk, acc[17]);
    acc[18] = fma(D82, mk, acc[18]);
    acc[19] = fma(D83, mk, acc[19]);
  }
  { const T mk = Mb[19];
    acc[0] = fma(D20, mk, acc[0]);
    acc[1] = fma(D35, mk, acc[1]);
    acc[2] = fma(D36, mk, acc[2]);
    acc[3] = fma(D37, mk, acc[3]);
    acc[4] = fma(D56, mk, acc[4]);
    acc[5] = fma(D57, mk, acc[5]);
    acc[6] = fma(D58, mk, acc[6]);
    acc[7] = fma(D59, mk, acc[7]);
    acc[8] = fma(D60, mk, acc[8]);
    acc[9] = fma(D61, mk, acc[9]);
  }
  { const T mk = Mb[20];
    acc[0] = fma(D21, mk, acc[0]);
    acc[1] = fma(D36, mk, acc[1]);
    acc[2] = fma(D38, mk, acc[2]);
    acc[3] = fma(D39, mk, acc[3]);
    acc[4] = fma(D57, mk, acc[4]);
    acc[5] = fma(D59, mk, acc[5]);
    acc[6] = fma(D60, mk, acc[6]);
    acc[7] = fma(D62, mk, acc[7]);
    acc[8] = fma(D63, mk, acc[8]);
    acc[9] = fma(D64, mk, acc[9]);
  }
  { const T mk = Mb[21];
    acc[0] = fma(D22, mk, acc[0]);
    acc[1] = fma(D37, mk, acc[1]);
    acc[2] = fma(D39, mk, acc[2]);
    acc[3] = fma(D40, mk, acc[3]);
    acc[4] = fma(D58, mk, acc[4]);
    acc[5] = fma(D60, mk, acc[5]);
    acc[6] = fma(D61, mk, acc[6]);
    acc[7] = fma(D63, mk, acc[7]);
    acc[8] = fma(D64, mk, acc[8]);
    acc[9] = fma(D65, mk, acc[9]);
  }
  { const T mk = Mb[22];
    acc[0] = fma(D23, mk, acc[0]);
    acc[1] = fma(D38, mk, acc[1]);
    acc[2] = fma(D41, mk, acc[2]);
    acc[3] = fma(D42, mk, acc[3]);
    acc[4] = fma(D59, mk, acc[4]);
    acc[5] = fma(D62, mk, acc[5]);
    acc[6] = fma(D63, mk, acc[6]);
    acc[7] = fma(D66, mk, acc[7]);
    acc[8] = fma(D67, mk, acc[8]);
    acc[9] = fma(D68, mk, acc[9]);
  }
  { const T mk = Mb[23];
    acc[0] = fma(D24, mk, acc[0]);
    acc[1] = fma(D39, mk, acc[1]);
    acc[2] = fma(D42, mk, acc[2]);
    acc[3] = fma(D43, mk, acc[3]);
    acc[4] = fma(D60, mk, acc[4]);
    acc[5] = fma(D63, mk, acc[5]);
    acc[6] = fma(D64, mk, acc[6]);
    acc[7] = fma(D67, mk, acc[7]);
    acc[8] = fma(D68, mk, acc[8]);
    acc[9] = fma(D69, mk, acc[9]);
  }
  { const T mk = Mb[24];
    acc[0] = fma(D25, mk, acc[0]);
    acc[1] = fma(D40, mk, acc[1]);
    acc[2] = fma(D43, mk, acc[2]);
    acc[3] = fma(D44, mk, acc[3]);
    acc[4] = fma(D61, mk, acc[4]);
    acc[5] = fma(D64, mk, acc[5]);
    acc[6] = fma(D65, mk, acc[6]);
    acc[7] = fma(D68, mk, acc[7]);
    acc[8] = fma(D69, mk, acc[8]);
    acc[9] = fma(D70, mk, acc[9]);
  }
  { const T mk = Mb[25];
    acc[0] = fma(D26, mk, acc[0]);
    acc[1] = fma(D41, mk, acc[1]);
    acc[2] = fma(D45, mk, acc[2]);
    acc[3] = fma(D46, mk, acc[3]);
    acc[4] = fma(D62, mk, acc[4]);
    acc[5] = fma(D66, mk, acc[5]);
    acc[6] = fma(D67, mk, acc[6]);
    acc[7] = fma(D71, mk, acc[7]);
    acc[8] = fma(D72, mk, acc[8]);
    acc[9] = fma(D73, mk, acc[9]);
  }
  { const T mk = Mb[26];
    acc[0] = fma(D27, mk, acc[0]);
    acc[1] = fma(D42, mk, acc[1]);
    acc[2] = fma(D46, mk, acc[2]);
    acc[3] = fma(D47, mk, acc[3]);
    acc[4] = fma(D63, mk, acc[4]);
    acc[5] = fma(D67, mk, acc[5]);
    acc[6] = fma(D68, mk, acc[6]);
    acc[7] = fma(D72, mk, acc[7]);
    acc[8] = fma(D73, mk, acc[8]);
    acc[9] = fma(D74, mk, acc[9]);
  }
  { const T mk = Mb[27];
    acc[0] = fma(D28, mk, acc[0]);
    acc[1] = fma(D43, mk, acc[1]);
    acc[2] = fma(D47, mk, acc[2]);
    acc[3] = fma(D48, mk, acc[3]);
    acc[4] = fma(D64, mk, acc[4]);
    acc[5] = fma(D68, mk, acc[5]);
    acc[6] = fma(D69, mk, acc[6]);
    acc[7] = fma(D73, mk, acc[7]);
    acc[8] = fma(D74, mk, acc[8]);
    acc[9] = fma(D75, mk, acc[9]);
  }
  { const T mk = Mb[28];
    acc[0] = fma(D29, mk, acc[0]);
    acc[1] = fma(D44, mk, acc[1]);
    acc[2] = fma(D48, mk, acc[2]);
    acc[3] = fma(D49, mk, acc[3]);
    acc[4] = fma(D65, mk, acc[4]);
    acc[5] = fma(D69, mk, acc[5]);
    acc[6] = fma(D70, mk, acc[6]);
    acc[7] = fma(D74, mk, acc[7]);
    acc[8] = fma(D75, mk, acc[8]);
    acc[9] = fma(D76, mk, acc[9]);
  }
  { const T mk = Mb[29];
    acc[0] = fma(D30, mk, acc[0]);
    acc[1] = fma(D45, mk, acc[1]);
    acc[2] = fma(D50, mk, acc[2]);
    acc[3] = fma(D51, mk, acc[3]);
    acc[4] = fma(D66, mk, acc[4]);
    acc[5] = fma(D71, mk, acc[5]);
    acc[6] = fma(D72, mk, acc[6]);
    acc[7] = fma(D77, mk, acc[7]);
    acc[8] = fma(D78, mk, acc[8]);
    acc[9] = fma(D79, mk, acc[9]);
  }
  { const T mk = Mb[30];
    acc[0] = fma(D31, mk, acc[0]);
    acc[1] = fma(D46, mk, acc[1]);
    acc[2] = fma(D51, mk, acc[2]);
    acc[3] = fma(D52, mk, acc[3]);
    acc[4] = fma(D67, mk, acc[4]);
    acc[5] = fma(D72, mk, acc[5]);
    acc[6] = fma(D73, mk, acc[6]);
    acc[7] = fma(D78, mk, acc[7]);
    acc[8] = fma(D79, mk, acc[8]);
    acc[9] = fma(D80, mk, acc[9]);
  }
  { const T mk = Mb[31];
    acc[0] = fma(D32, mk, acc[0]);
    acc[1] = fma(D47, mk, acc[1]);
    acc[2] = fma(D52, mk, acc[2]);
    acc[3] = fma(D53, mk, acc[3]);
    acc[4] = fma(D68, mk, acc[4]);
    acc[5] = fma(D73, mk, acc[5]);
    acc[6] = fma(D74, mk, acc[6]);
    acc[7] = fma(D79, mk, acc[7]);
    acc[8] = fma(D80, mk, acc[8]);
    acc[9] = fma(D81, mk, acc[9]);
  }
  { const T mk = Mb[32];
    acc[0] = fma(D33, mk, acc[0]);
    acc[1] = fma(D48, mk, acc[1]);
    acc[2] = fma(D53, mk, acc[2]);
    acc[3] = fma(D54, mk, acc[3]);
    acc[4] = fma(D69, mk, acc[4]);
    acc[5] = fma(D74, mk, acc[5]);
    acc[6] = fma(D75, mk, acc[6]);
    acc[7] = fma(D80, mk, acc[7]);
    acc[8] = fma(D81, mk, acc[8]);
    acc[9] = fma(D82, mk, acc[9]);
  }
  { const T mk = Mb[33];
    acc[0] = fma(D34, mk, acc[0]);
    acc[1] = fma(D49, mk, acc[1]);
    acc[2] = fma(D54, mk, acc[2]);
    acc[3] = fma(D55, mk, acc[3]);
    acc[4] = fma(D70, mk, acc[4]);
    acc[5] = fma(D75, mk, acc[5]);
    acc[6] = fma(D76, mk, acc[6]);
    acc[7] = fma(D81, mk, acc[7]);
    acc[8] = fma(D82, mk, acc[8]);
    acc[9] = fma(D83, mk, acc[9]);
  }
  { const T mk = Mb[34];
    acc[0] = fma(D35, mk, acc[0]);
    acc[1] = fma(D56, mk, acc[1]);
    acc[2] = fma(D57, mk, acc[2]);
    acc[3] = fma(D58, mk, acc[3]);
  }
  { const T mk = Mb[35];
    acc[0] = fma(D36, mk, acc[0]);
    acc[1] = fma(D57, mk, acc[1]);
    acc[2] = fma(D59, mk, acc[2]);
    acc[3] = fma(D60, mk, acc[3]);
  }
  { const T mk = Mb[36];
    acc[0] = fma(D37, mk, acc[0]);
    acc[1] = fma(D58, mk, acc[1]);
    acc[2] = fma(D60, mk, acc[2]);
    acc[3] = fma(D61, mk, acc[3]);
  }
  { const T mk = Mb[37];
    acc[0] = fma(D38, mk, acc[0]);
    acc[1] = fma(D59, mk, acc[1]);
    acc[2] = fma(D62, mk, acc[2]);
    acc[3] = fma(D63, mk, acc[3]);
  }
  { const T mk = Mb[38];
    acc[0] = fma(D39, mk, acc[0]);
    acc[1] = fma(D60, mk, acc[1]);
    acc[2] = fma(D63, mk, acc[2]);
    acc[3] = fma(D64, mk, acc[3]);
  }
  { const T mk = Mb[39];
    acc[0] = fma(D40, mk, acc[0]);
    acc[1] = fma(D61, mk, acc[1]);
    acc[2] = fma(D64, mk, acc[2]);
    acc[3] = fma(D65, mk, acc[3]);
  }
  { const T mk = Mb[40];
    acc[0] = fma(D41, mk, acc[0]);
    acc[1] = fma(D62, mk, acc[1]);
    acc[2] = fma(D66, mk, acc[2]);
    acc[3] = fma(D67, mk, acc[3]);
  }
  { const T mk = Mb[41];
    acc[0] = fma(D42, mk, acc[0]);
    acc[1] = fma(D63, mk, acc[1]);
    acc[2] = fma(D67, mk, acc[2]);
    acc[3] = fma(D68, mk, acc[3]);
  }
  { const T mk = Mb[42];
    acc[0] = fma(D43, mk, acc[0]);
    acc[1] = fma(D64, mk, acc[1]);
    acc[2] = fma(D68, mk, acc[2]);
    acc[3] = fma(D69, mk, acc[3]);
  }
  { const T mk = Mb[43];
    acc[0] = fma(D44, mk, acc[0]);
    acc[1] = fma(D65, mk, acc[1]);
    acc[2] = fma(D69, mk, acc[2]);
    acc[3] = fma(D70, mk, acc[3]);
  }
  { const T mk = Mb[44];
    acc[0] = fma(D45, mk, acc[0]);
    acc[1] = fma(D66, mk, acc[1]);
    acc[2] = fma(D71, mk, acc[2]);
    acc[3] = fma(D72, mk, acc[3]);
  }
  { const T mk = Mb[45];
    acc[0] = fma(D46, mk, acc[0]);
    acc[1] = fma(D67, mk, acc[1]);
    acc[2] = fma(D72, mk, acc[2]);
    acc[3] = fma(D73, mk, acc[3]);
  }
  { const T mk = Mb[46];
    acc[0] = fma(D47, mk, acc[0]);
    acc[1] = fma(D68, mk, acc[1]);
    acc[2] = fma(D73, mk, acc[2]);
    acc[3] = fma(D74, mk, acc[3]);
  }
  { const T mk = Mb[47];
    acc[0] = fma(D48, mk, acc[0]);
    acc[1] = fma(D69, mk, acc[1]);
    acc[2] = fma(D74, mk, acc[2]);
    acc[3] = fma(D75, mk, acc[3]);
  }
  { const T mk = Mb[48];
    acc[0] = fma(D49, mk, acc[0]);
    acc[1] = fma(D70, mk, acc[1]);
    acc[2] = fma(D75, mk, acc[2]);
    acc[3] = fma(D76, mk, acc[3]);
  }
  { const T mk = Mb[49];
    acc[0] = fma(D50, mk, acc[0]);
    acc[1] = fma(D71, mk, acc[1]);
    acc[2] = fma(D77, mk, acc[2]);
    acc[3] = fma(D78, mk, acc[3]);
  }
  { const T mk = Mb[50];
    acc[0] = fma(D51, mk, acc[0]);
    acc[1] = fma(D72, mk, acc[1]);
    acc[2] = fma(D78, mk, acc[2]);
    acc[3] = fma(D79, mk, acc[3]);
  }
  { const T mk = Mb[51];
    acc[0] = fma(D52, mk, acc[0]);
    acc[1] = fma(D73, mk, acc[1]);
    acc[2] = fma(D79, mk, acc[2]);
    acc[3] = fma(D80, mk, acc[3]);
  }
  { const T mk = Mb[52];
    acc[0] = fma(D53, mk, acc[0]);
    acc[1] = fma(D74, mk, acc[1]);
    acc[2] = fma(D80, mk, acc[2]);
    acc[3] = fma(D81, mk, acc[3]);
  }
  { const T mk = Mb[53];
    acc[0] = fma(D54, mk, acc[0]);
    acc[1] = fma(D75, mk, acc[1]);
    acc[2] = fma(D81, mk, acc[2]);
    acc[3] = fma(D82, mk, acc[3]);
  }
  { const T mk = Mb[54];
    acc[0] = fma(D55, mk, acc[0]);
    acc[1] = fma(D76, mk, acc[1]);
    acc[2] = fma(D82, mk, acc[2]);
    acc[3] = fma(D83, mk, acc[3]);
  }
  { const T mk = Mb[55];
    acc[0] = fma(D56, mk, acc[0]);
  }
  { const T mk = Mb[56];
    acc[0] = fma(D57, mk, acc[0]);
  }
  { const T mk = Mb[57];
    acc[0] = fma(D58, mk, acc[0]);
  }
  { const T mk = Mb[58];
    acc[0] = fma(D59, mk, acc[0]);
  }
  { const T mk = Mb[59];
    acc[0] = fma(D60, mk, acc[0]);
  }
  { const T mk = Mb[60];
    acc[0] = fma(D61, mk, acc[0]);
  }
  { const T mk = Mb[61];
    acc[0] = fma(D62, mk, acc[0]);
  }
  { const T mk = Mb[62];
    acc[0] = fma(D63, mk, acc[0]);
  }
  { const T mk = Mb[63];
    acc[0] = fma(D64, mk, acc[0]);
  }
  { const T mk = Mb[64];
    acc[0] = fma(D65, mk, acc[0]);
  }
  { const T mk = Mb[65];
    acc[0] = fma(D66, mk, acc[0]);
  }
  { const T mk = Mb[66];
    acc[0] = fma(D67, mk, acc[0]);
  }
  { const T mk = Mb[67];
    acc[0] = fma(D68, mk, acc[0]);
  }
  { const T mk = Mb[68];
    acc[0] = fma(D69, mk, acc[0]);
  }
  { const T mk = Mb[69];
    acc[0] = fma(D70, mk, acc[0]);
  }
  { const T mk = Mb[70];
    acc[0] = fma(D71, mk, acc[0]);
  }
  { const T mk = Mb[71];
    acc[0] = fma(D72, mk, acc[0]);
  }
  { const T mk = Mb[72];
    acc[0] = fma(D73, mk, acc[0]);
  }
  { const T mk = Mb[73];
    acc[0] = fma(D74, mk, acc[0]);
  }
  { const T mk = Mb[74];
    acc[0] = fma(D75, mk, acc[0]);
  }
  { const T mk = Mb[75];
    acc[0] = fma(D76, mk, acc[0]);
  }
  { const T mk = Mb[76];
    acc[0] = fma(D77, mk, acc[0]);
  }
  { const T mk = Mb[77];
    acc[0] = fma(D78, mk, acc[0]);
  }
  { const T mk = Mb[78];
    acc[0] = fma(D79, mk, acc[0]);
  }
  { const T mk = Mb[79];
    acc[0] = fma(D80, mk, acc[0]);
  }
  { const T mk = Mb[80];
    acc[0] = fma(D81, mk, acc[0]);
  }
  { const T mk = Mb[81];
    acc[0] = fma(D82, mk, acc[0]);
  }
  { const T mk = Mb[82];
    acc[0] = fma(D83, mk, acc[0]);
  }
}

// P2M of a dipole (s0, s1, s2) at offset (x, y, z) = centre - site, order 5
template <typename T>
__device__ __forceinline__ void p2m_m1_p5(T x, T y, T z, T s0, T s1, T s2, T* __restrict__ acc) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  { const T v = s0;
    acc[0] = fma(T(1), v, acc[0]);
    acc[3] = fma(px1, v, acc[3]);
    acc[4] = fma(py1, v, acc[4]);
    acc[5] = fma(pz1, v, acc[5]);
    acc[9] = fma(px2, v, acc[9]);
    acc[10] = fma(m_1_1_0, v, acc[10]);
    acc[11] = fma(m_1_0_1, v, acc[11]);
    acc[12] = fma(py2, v, acc[12]);
    acc[13] = fma(m_0_1_1, v, acc[13]);
    acc[14] = fma(pz2, v, acc[14]);
    acc[19] = fma(px3, v, acc[19]);
    acc[20] = fma(m_2_1_0, v, acc[20]);
    acc[21] = fma(m_2_0_1, v, acc[21]);
    acc[22] = fma(m_1_2_0, v, acc[22]);
    acc[23] = fma(m_1_1_1, v, acc[23]);
    acc[24] = fma(m_1_0_2, v, acc[24]);
    acc[25] = fma(py3, v, acc[25]);
    acc[26] = fma(m_0_2_1, v, acc[26]);
    acc[27] = fma(m_0_1_2, v, acc[27]);
    acc[28] = fma(pz3, v, acc[28]);
    acc[34] = fma(px4, v, acc[34]);
    acc[35] = fma(m_3_1_0, v, acc[35]);
    acc[36] = fma(m_3_0_1, v, acc[36]);
    acc[37] = fma(m_2_2_0, v, acc[37]);
    acc[38] = fma(m_2_1_1, v, acc[38]);
    acc[39] = fma(m_2_0_2, v, acc[39]);
    acc[40] = fma(m_1_3_0, v, acc[40]);
    acc[41] = fma(m_1_2_1, v, acc[41]);
    acc[42] = fma(m_1_1_2, v, acc[42]);
    acc[43] = fma(m_1_0_3, v, acc[43]);
    acc[44] = fma(py4, v, acc[44]);
    acc[45] = fma(m_0_3_1, v, acc[45]);
    acc[46] = fma(m_0_2_2, v, acc[46]);
    acc[47] = fma(m_0_1_3, v, acc[47]);
    acc[48] = fma(pz4, v, acc[48]);
  }
  { const T v = s1;
    acc[1] = fma(T(1), v, acc[1]);
    acc[4] = fma(px1, v, acc[4]);
    acc[6] = fma(py1, v, acc[6]);
    acc[7] = fma(pz1, v, acc[7]);
    acc[10] = fma(px2, v, acc[10]);
    acc[12] = fma(m_1_1_0, v, acc[12]);
    acc[13] = fma(m_1_0_1, v, acc[13]);
    acc[15] = fma(py2, v, acc[15]);
    acc[16] = fma(m_0_1_1, v, acc[16]);
    acc[17] = fma(pz2, v, acc[17]);
    acc[20] = fma(px3, v, acc[20]);
    acc[22] = fma(m_2_1_0, v, acc[22]);
    acc[23] = fma(m_2_0_1, v, acc[23]);
    acc[25] = fma(m_1_2_0, v, acc[25]);
    acc[26] = fma(m_1_1_1, v, acc[26]);
    acc[27] = fma(m_1_0_2, v, acc[27]);
    acc[29] = fma(py3, v, acc[29]);
    acc[30] = fma(m_0_2_1, v, acc[30]);
    acc[31] = fma(m_0_1_2, v, acc[31]);
    acc[32] = fma(pz3, v, acc[32]);
    acc[35] = fma(px4, v, acc[35]);
    acc[37] = fma(m_3_1_0, v, acc[37]);
    acc[38] = fma(m_3_0_1, v, acc[38]);
    acc[40] = fma(m_2_2_0, v, acc[40]);
    acc[41] = fma(m_2_1_1, v, acc[41]);
    acc[42] = fma(m_2_0_2, v, acc[42]);
    acc[44] = fma(m_1_3_0, v, acc[44]);
    acc[45] = fma(m_1_2_1, v, acc[45]);
    acc[46] = fma(m_1_1_2, v, acc[46]);
    acc[47] = fma(m_1_0_3, v, acc[47]);
    acc[49] = fma(py4, v, acc[49]);
    acc[50] = fma(m_0_3_1, v, acc[50]);
    acc[51] = fma(m_0_2_2, v, acc[51]);
    acc[52] = fma(m_0_1_3, v, acc[52]);
    acc[53] = fma(pz4, v, acc[53]);
  }
  { const T v = s2;
    acc[2] = fma(T(1), v, acc[2]);
    acc[5] = fma(px1, v, acc[5]);
    acc[7] = fma(py1, v, acc[7]);
    acc[8] = fma(pz1, v, acc[8]);
    acc[11] = fma(px2, v, acc[11]);
    acc[13] = fma(m_1_1_0, v, acc[13]);
    acc[14] = fma(m_1_0_1, v, acc[14]);
    acc[16] = fma(py2, v, acc[16]);
    acc[17] = fma(m_0_1_1, v, acc[17]);
    acc[18] = fma(pz2, v, acc[18]);
    acc[21] = fma(px3, v, acc[21]);
    acc[23] = fma(m_2_1_0, v, acc[23]);
    acc[24] = fma(m_2_0_1, v, acc[24]);
    acc[26] = fma(m_1_2_0, v, acc[26]);
    acc[27] = fma(m_1_1_1, v, acc[27]);
    acc[28] = fma(m_1_0_2, v, acc[28]);
    acc[30] = fma(py3, v, acc[30]);
    acc[31] = fma(m_0_2_1, v, acc[31]);
    acc[32] = fma(m_0_1_2, v, acc[32]);
    acc[33] = fma(pz3, v, acc[33]);
    acc[36] = fma(px4, v, acc[36]);
    acc[38] = fma(m_3_1_0, v, acc[38]);
    acc[39] = fma(m_3_0_1, v, acc[39]);
    acc[41] = fma(m_2_2_0, v, acc[41]);
    acc[42] = fma(m_2_1_1, v, acc[42]);
    acc[43] = fma(m_2_0_2, v, acc[43]);
    acc[45] = fma(m_1_3_0, v, acc[45]);
    acc[46] = fma(m_1_2_1, v, acc[46]);
    acc[47] = fma(m_1_1_2, v, acc[47]);
    acc[48] = fma(m_1_0_3, v, acc[48]);
    acc[50] = fma(py4, v, acc[50]);
    acc[51] = fma(m_0_3_1, v, acc[51]);
    acc[52] = fma(m_0_2_2, v, acc[52]);
    acc[53] = fma(m_0_1_3, v, acc[53]);
    acc[54] = fma(pz4, v, acc[54]);
  }
}
// M2M: multipole Mc about a centre at (x, y, z) from this one, order 5
template <typename T>
__device__ __forceinline__ void m2m_m1_p5(T x, T y, T z, const T* __restrict__ Mc, T* __restrict__ acc) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  { const T v = Mc[0];
    acc[0] = fma(T(1), v, acc[0]);
    acc[3] = fma(px1, v, acc[3]);
    acc[4] = fma(py1, v, acc[4]);
    acc[5] = fma(pz1, v, acc[5]);
    acc[9] = fma(px2, v, acc[9]);
    acc[10] = fma(m_1_1_0, v, acc[10]);
    acc[11] = fma(m_1_0_1, v, acc[11]);
    acc[12] = fma(py2, v, acc[12]);
    acc[13] = fma(m_0_1_1, v, acc[13]);
    acc[14] = fma(pz2, v, acc[14]);
    acc[19] = fma(px3, v, acc[19]);
    acc[20] = fma(m_2_1_0, v, acc[20]);
    acc[21] = fma(m_2_0_1, v, acc[21]);
    acc[22] = fma(m_1_2_0, v, acc[22]);
    acc[23] = fma(m_1_1_1, v, acc[23]);
    acc[24] = fma(m_1_0_2, v, acc[24]);
    acc[25] = fma(py3, v, acc[25]);
    acc[26] = fma(m_0_2_1, v, acc[26]);
    acc[27] = fma(m_0_1_2, v, acc[27]);
    acc[28] = fma(pz3, v, acc[28]);
    acc[34] = fma(px4, v, acc[34]);
    acc[35] = fma(m_3_1_0, v, acc[35]);
    acc[36] = fma(m_3_0_1, v, acc[36]);
    acc[37] = fma(m_2_2_0, v, acc[37]);
    acc[38] = fma(m_2_1_1, v, acc[38]);
    acc[39] = fma(m_2_0_2, v, acc[39]);
    acc[40] = fma(m_1_3_0, v, acc[40]);
    acc[41] = fma(m_1_2_1, v, acc[41]);
    acc[42] = fma(m_1_1_2, v, acc[42]);
    acc[43] = fma(m_1_0_3, v, acc[43]);
    acc[44] = fma(py4, v, acc[44]);
    acc[45] = fma(m_0_3_1, v, acc[45]);
    acc[46] = fma(m_0_2_2, v, acc[46]);
    acc[47] = fma(m_0_1_3, v, acc[47]);
    acc[48] = fma(pz4, v, acc[48]);
  }
  { const T v = Mc[1];
    acc[1] = fma(T(1), v, acc[1]);
    acc[4] = fma(px1, v, acc[4]);
    acc[6] = fma(py1, v, acc[6]);
    acc[7] = fma(pz1, v, acc[7]);
    acc[10] = fma(px2, v, acc[10]);
    acc[12] = fma(m_1_1_0, v, acc[12]);
    acc[13] = fma(m_1_0_1, v, acc[13]);
    acc[15] = fma(py2, v, acc[15]);
    acc[16] = fma(m_0_1_1, v, acc[16]);
    acc[17] = fma(pz2, v, acc[17]);
    acc[20] = fma(px3, v, acc[20]);
    acc[22] = fma(m_2_1_0, v, acc[22]);
    acc[23] = fma(m_2_0_1, v, acc[23]);
    acc[25] = fma(m_1_2_0, v, acc[25]);
    acc[26] = fma(m_1_1_1, v, acc[26]);
    acc[27] = fma(m_1_0_2, v, acc[27]);
    acc[29] = fma(py3, v, acc[29]);
    acc[30] = fma(m_0_2_1, v, acc[30]);
    acc[31] = fma(m_0_1_2, v, acc[31]);
    acc[32] = fma(pz3, v, acc[32]);
    acc[35] = fma(px4, v, acc[35]);
    acc[37] = fma(m_3_1_0, v, acc[37]);
    acc[38] = fma(m_3_0_1, v, acc[38]);
    acc[40] = fma(m_2_2_0, v, acc[40]);
    acc[41] = fma(m_2_1_1, v, acc[41]);
    acc[42] = fma(m_2_0_2, v, acc[42]);
    acc[44] = fma(m_1_3_0, v, acc[44]);
    acc[45] = fma(m_1_2_1, v, acc[45]);
    acc[46] = fma(m_1_1_2, v, acc[46]);
    acc[47] = fma(m_1_0_3, v, acc[47]);
    acc[49] = fma(py4, v, acc[49]);
    acc[50] = fma(m_0_3_1, v, acc[50]);
    acc[51] = fma(m_0_2_2, v, acc[51]);
    acc[52] = fma(m_0_1_3, v, acc[52]);
    acc[53] = fma(pz4, v, acc[53]);
  }
  { const T v = Mc[2];
    acc[2] = fma(T(1), v, acc[2]);
    acc[5] = fma(px1, v, acc[5]);
    acc[7] = fma(py1, v, acc[7]);
    acc[8] = fma(pz1, v, acc[8]);
    acc[11] = fma(px2, v, acc[11]);
    acc[13] = fma(m_1_1_0, v, acc[13]);
    acc[14] = fma(m_1_0_1, v, acc[14]);
    acc[16] = fma(py2, v, acc[16]);
    acc[17] = fma(m_0_1_1, v, acc[17]);
    acc[18] = fma(pz2, v, acc[18]);
    acc[21] = fma(px3, v, acc[21]);
    acc[23] = fma(m_2_1_0, v, acc[23]);
    acc[24] = fma(m_2_0_1, v, acc[24]);
    acc[26] = fma(m_1_2_0, v, acc[26]);
    acc[27] = fma(m_1_1_1, v, acc[27]);
    acc[28] = fma(m_1_0_2, v, acc[28]);
    acc[30] = fma(py3, v, acc[30]);
    acc[31] = fma(m_0_2_1, v, acc[31]);
    acc[32] = fma(m_0_1_2, v, acc[32]);
    acc[33] = fma(pz3, v, acc[33]);
    acc[36] = fma(px4, v, acc[36]);
    acc[38] = fma(m_3_1_0, v, acc[38]);
    acc[39] = fma(m_3_0_1, v, acc[39]);
    acc[41] = fma(m_2_2_0, v, acc[41]);
    acc[42] = fma(m_2_1_1, v, acc[42]);
    acc[43] = fma(m_2_0_2, v, acc[43]);
    acc[45] = fma(m_1_3_0, v, acc[45]);
    acc[46] = fma(m_1_2_1, v, acc[46]);
    acc[47] = fma(m_1_1_2, v, acc[47]);
    acc[48] = fma(m_1_0_3, v, acc[48]);
    acc[50] = fma(py4, v, acc[50]);
    acc[51] = fma(m_0_3_1, v, acc[51]);
    acc[52] = fma(m_0_2_2, v, acc[52]);
    acc[53] = fma(m_0_1_3, v, acc[53]);
    acc[54] = fma(pz4, v, acc[54]);
  }
  { const T v = Mc[3];
    acc[3] = fma(T(1), v, acc[3]);
    acc[9] = fma(px1, v, acc[9]);
    acc[10] = fma(py1, v, acc[10]);
    acc[11] = fma(pz1, v, acc[11]);
    acc[19] = fma(px2, v, acc[19]);
    acc[20] = fma(m_1_1_0, v, acc[20]);
    acc[21] = fma(m_1_0_1, v, acc[21]);
    acc[22] = fma(py2, v, acc[22]);
    acc[23] = fma(m_0_1_1, v, acc[23]);
    acc[24] = fma(pz2, v, acc[24]);
    acc[34] = fma(px3, v, acc[34]);
    acc[35] = fma(m_2_1_0, v, acc[35]);
    acc[36] = fma(m_2_0_1, v, acc[36]);
    acc[37] = fma(m_1_2_0, v, acc[37]);
    acc[38] = fma(m_1_1_1, v, acc[38]);
    acc[39] = fma(m_1_0_2, v, acc[39]);
    acc[40] = fma(py3, v, acc[40]);
    acc[41] = fma(m_0_2_1, v, acc[41]);
    acc[42] = fma(m_0_1_2, v, acc[42]);
    acc[43] = fma(pz3, v, acc[43]);
  }
  { const T v = Mc[4];
    acc[4] = fma(T(1), v, acc[4]);
    acc[10] = fma(px1, v, acc[10]);
    acc[12] = fma(py1, v, acc[12]);
    acc[13] = fma(pz1, v, acc[13]);
    acc[20] = fma(px2, v, acc[20]);
    acc[22] = fma(m_1_1_0, v, acc[22]);
    acc[23] = fma(m_1_0_1, v, acc[23]);
    acc[25] = fma(py2, v, acc[25]);
    acc[26] = fma(m_0_1_1, v, acc[26]);
    acc[27] = fma(pz2, v, acc[27]);
    acc[35] = fma(px3, v, acc[35]);
    acc[37] = fma(m_2_1_0, v, acc[37]);
    acc[38] = fma(m_2_0_1, v, acc[38]);
    acc[40] = fma(m_1_2_0, v, acc[40]);
    acc[41] = fma(m_1_1_1, v, acc[41]);
    acc[42] = fma(m_1_0_2, v, acc[42]);
    acc[44] = fma(py3, v, acc[44]);
    acc[45] = fma(m_0_2_1, v, acc[45]);
    acc[46] = fma(m_0_1_2, v, acc[46]);
    acc[47] = fma(pz3, v, acc[47]);
  }
  { const T v = Mc[5];
    acc[5] = fma(T(1), v, acc[5]);
    acc[11] = fma(px1, v, acc[11]);
    acc[13] = fma(py1, v, acc[13]);
    acc[14] = fma(pz1, v, acc[14]);
    acc[21] = fma(px2, v, acc[21]);
    acc[23] = fma(m_1_1_0, v, acc[23]);
    acc[24] = fma(m_1_0_1, v, acc[24]);
    acc[26] = fma(py2, v, acc[26]);
    acc[27] = fma(m_0_1_1, v, acc[27]);
    acc[28] = fma(pz2, v, acc[28]);
    acc[36] = fma(px3, v, acc[36]);
    acc[38] = fma(m_2_1_0, v, acc[38]);
    acc[39] = fma(m_2_0_1, v, acc[39]);
    acc[41] = fma(m_1_2_0, v, acc[41]);
    acc[42] = fma(m_1_1_1, v, acc[42]);
    acc[43] = fma(m_1_0_2, v, acc[43]);
    acc[45] = fma(py3, v, acc[45]);
    acc[46] = fma(m_0_2_1, v, acc[46]);
    acc[47] = fma(m_0_1_2, v, acc[47]);
    acc[48] = fma(pz3, v, acc[48]);
  }
  { const T v = Mc[6];
    acc[6] = fma(T(1), v, acc[6]);
    acc[12] = fma(px1, v, acc[12]);
    acc[15] = fma(py1, v, acc[15]);
    acc[16] = fma(pz1, v, acc[16]);
    acc[22] = fma(px2, v, acc[22]);
    acc[25] = fma(m_1_1_0, v, acc[25]);
    acc[26] = fma(m_1_0_1, v, acc[26]);
    acc[29] = fma(py2, v, acc[29]);
    acc[30] = fma(m_0_1_1, v, acc[30]);
    acc[31] = fma(pz2, v, acc[31]);
    acc[37] = fma(px3, v, acc[37]);
    acc[40] = fma(m_2_1_0, v, acc[40]);
    acc[41] = fma(m_2_0_1, v, acc[41]);
    acc[44] = fma(m_1_2_0, v, acc[44]);
    acc[45] = fma(m_1_1_1, v, acc[45]);
    acc[46] = fma(m_1_0_2, v, acc[46]);
    acc[49] = fma(py3, v, acc[49]);
    acc[50] = fma(m_0_2_1, v, acc[50]);
    acc[51] = fma(m_0_1_2, v, acc[51]);
    acc[52] = fma(pz3, v, acc[52]);
  }
  { const T v = Mc[7];
    acc[7] = fma(T(1), v, acc[7]);
    acc[13] = fma(px1, v, acc[13]);
    acc[16] = fma(py1, v, acc[16]);
    acc[17] = fma(pz1, v, acc[17]);
    acc[23] = fma(px2, v, acc[23]);
    acc[26] = fma(m_1_1_0, v, acc[26]);
    acc[27] = fma(m_1_0_1, v, acc[27]);
    acc[30] = fma(py2, v, acc[30]);
    acc[31] = fma(m_0_1_1, v, acc[31]);
    acc[32] = fma(pz2, v, acc[32]);
    acc[38] = fma(px3, v, acc[38]);
    acc[41] = fma(m_2_1_0, v, acc[41]);
    acc[42] = fma(m_2_0_1, v, acc[42]);
    acc[45] = fma(m_1_2_0, v, acc[45]);
    acc[46] = fma(m_1_1_1, v, acc[46]);
    acc[47] = fma(m_1_0_2, v, acc[47]);
    acc[50] = fma(py3, v, acc[50]);
    acc[51] = fma(m_0_2_1, v, acc[51]);
    acc[52] = fma(m_0_1_2, v, acc[52]);
    acc[53] = fma(pz3, v, acc[53]);
  }
  { const T v = Mc[8];
    acc[8] = fma(T(1), v, acc[8]);
    acc[14] = fma(px1, v, acc[14]);
    acc[17] = fma(py1, v, acc[17]);
    acc[18] = fma(pz1, v, acc[18]);
    acc[24] = fma(px2, v, acc[24]);
    acc[27] = fma(m_1_1_0, v, acc[27]);
    acc[28] = fma(m_1_0_1, v, acc[28]);
    acc[31] = fma(py2, v, acc[31]);
    acc[32] = fma(m_0_1_1, v, acc[32]);
    acc[33] = fma(pz2, v, acc[33]);
    acc[39] = fma(px3, v, acc[39]);
    acc[42] = fma(m_2_1_0, v, acc[42]);
    acc[43] = fma(m_2_0_1, v, acc[43]);
    acc[46] = fma(m_1_2_0, v, acc[46]);
    acc[47] = fma(m_1_1_1, v, acc[47]);
    acc[48] = fma(m_1_0_2, v, acc[48]);
    acc[51] = fma(py3, v, acc[51]);
    acc[52] = fma(m_0_2_1, v, acc[52]);
    acc[53] = fma(m_0_1_2, v, acc[53]);
    acc[54] = fma(pz3, v, acc[54]);
  }
  { const T v = Mc[9];
    acc[9] = fma(T(1), v, acc[9]);
    acc[19] = fma(px1, v, acc[19]);
    acc[20] = fma(py1, v, acc[20]);
    acc[21] = fma(pz1, v, acc[21]);
    acc[34] = fma(px2, v, acc[34]);
    acc[35] = fma(m_1_1_0, v, acc[35]);
    acc[36] = fma(m_1_0_1, v, acc[36]);
    acc[37] = fma(py2, v, acc[37]);
    acc[38] = fma(m_0_1_1, v, acc[38]);
    acc[39] = fma(pz2, v, acc[39]);
  }
  { const T v = Mc[10];
    acc[10] = fma(T(1), v, acc[10]);
    acc[20] = fma(px1, v, acc[20]);
    acc[22] = fma(py1, v, acc[22]);
    acc[23] = fma(pz1, v, acc[23]);
    acc[35] = fma(px2, v, acc[35]);
    acc[37] = fma(m_1_1_0, v, acc[37]);
    acc[38] = fma(m_1_0_1, v, acc[38]);
    acc[40] = fma(py2, v, acc[40]);
    acc[41] = fma(m_0_1_1, v, acc[41]);
    acc[42] = fma(pz2, v, acc[42]);
  }
  { const T v = Mc[11];
    acc[11] = fma(T(1), v, acc[11]);
    acc[21] = fma(px1, v, acc[21]);
    acc[23] = fma(py1, v, acc[23]);
    acc[24] = fma(pz1, v, acc[24]);
    acc[36] = fma(px2, v, acc[36]);
    acc[38] = fma(m_1_1_0, v, acc[38]);
    acc[39] = fma(m_1_0_1, v, acc[39]);
    acc[41] = fma(py2, v, acc[41]);
    acc[42] = fma(m_0_1_1, v, acc[42]);
    acc[43] = fma(pz2, v, acc[43]);
  }
  { const T v = Mc[12];
    acc[12] = fma(T(1), v, acc[12]);
    acc[22] = fma(px1, v, acc[22]);
    acc[25] = fma(py1, v, acc[25]);
    acc[26] = fma(pz1, v, acc[26]);
    acc[37] = fma(px2, v, acc[37]);
    acc[40] = fma(m_1_1_0, v, acc[40]);
    acc[41] = fma(m_1_0_1, v, acc[41]);
    acc[44] = fma(py2, v, acc[44]);
    acc[45] = fma(m_0_1_1, v, acc[45]);
    acc[46] = fma(pz2, v, acc[46]);
  }
  { const T v = Mc[13];
    acc[13] = fma(T(1), v, acc[13]);
    acc[23] = fma(px1, v, acc[23]);
    acc[26] = fma(py1, v, acc[26]);
    acc[27] = fma(pz1, v, acc[27]);
    acc[38] = fma(px2, v, acc[38]);
    acc[41] = fma(m_1_1_0, v, acc[41]);
    acc[42] = fma(m_1_0_1, v, acc[42]);
    acc[45] = fma(py2, v, acc[45]);
    acc[46] = fma(m_0_1_1, v, acc[46]);
    acc[47] = fma(pz2, v, acc[47]);
  }
  { const T v = Mc[14];
    acc[14] = fma(T(1), v, acc[14]);
    acc[24] = fma(px1, v, acc[24]);
    acc[27] = fma(py1, v, acc[27]);
    acc[28] = fma(pz1, v, acc[28]);
    acc[39] = fma(px2, v, acc[39]);
    acc[42] = fma(m_1_1_0, v, acc[42]);
    acc[43] = fma(m_1_0_1, v, acc[43]);
    acc[46] = fma(py2, v, acc[46]);
    acc[47] = fma(m_0_1_1, v, acc[47]);
    acc[48] = fma(pz2, v, acc[48]);
  }
  { const T v = Mc[15];
    acc[15] = fma(T(1), v, acc[15]);
    acc[25] = fma(px1, v, acc[25]);
    acc[29] = fma(py1, v, acc[29]);
    acc[30] = fma(pz1, v, acc[30]);
    acc[40] = fma(px2, v, acc[40]);
    acc[44] = fma(m_1_1_0, v, acc[44]);
    acc[45] = fma(m_1_0_1, v, acc[45]);
    acc[49] = fma(py2, v, acc[49]);
    acc[50] = fma(m_0_1_1, v, acc[50]);
    acc[51] = fma(pz2, v, acc[51]);
  }
  { const T v = Mc[16];
    acc[16] = fma(T(1), v, acc[16]);
    acc[26] = fma(px1, v, acc[26]);
    acc[30] = fma(py1, v, acc[30]);
    acc[31] = fma(pz1, v, acc[31]);
    acc[41] = fma(px2, v, acc[41]);
    acc[45] = fma(m_1_1_0, v, acc[45]);
    acc[46] = fma(m_1_0_1, v, acc[46]);
    acc[50] = fma(py2, v, acc[50]);
    acc[51] = fma(m_0_1_1, v, acc[51]);
    acc[52] = fma(pz2, v, acc[52]);
  }
  { const T v = Mc[17];
    acc[17] = fma(T(1), v, acc[17]);
    acc[27] = fma(px1, v, acc[27]);
    acc[31] = fma(py1, v, acc[31]);
    acc[32] = fma(pz1, v, acc[32]);
    acc[42] = fma(px2, v, acc[42]);
    acc[46] = fma(m_1_1_0, v, acc[46]);
    acc[47] = fma(m_1_0_1, v, acc[47]);
    acc[51] = fma(py2, v, acc[51]);
    acc[52] = fma(m_0_1_1, v, acc[52]);
    acc[53] = fma(pz2, v, acc[53]);
  }
  { const T v = Mc[18];
    acc[18] = fma(T(1), v, acc[18]);
    acc[28] = fma(px1, v, acc[28]);
    acc[32] = fma(py1, v, acc[32]);
    acc[33] = fma(pz1, v, acc[33]);
    acc[43] = fma(px2, v, acc[43]);
    acc[47] = fma(m_1_1_0, v, acc[47]);
    acc[48] = fma(m_1_0_1, v, acc[48]);
    acc[52] = fma(py2, v, acc[52]);
    acc[53] = fma(m_0_1_1, v, acc[53]);
    acc[54] = fma(pz2, v, acc[54]);
  }
  { const T v = Mc[19];
    acc[19] = fma(T(1), v, acc[19]);
    acc[34] = fma(px1, v, acc[34]);
    acc[35] = fma(py1, v, acc[35]);
    acc[36] = fma(pz1, v, acc[36]);
  }
  { const T v = Mc[20];
    acc[20] = fma(T(1), v, acc[20]);
    acc[35] = fma(px1, v, acc[35]);
    acc[37] = fma(py1, v, acc[37]);
    acc[38] = fma(pz1, v, acc[38]);
  }
  { const T v = Mc[21];
    acc[21] = fma(T(1), v, acc[21]);
    acc[36] = fma(px1, v, acc[36]);
    acc[38] = fma(py1, v, acc[38]);
    acc[39] = fma(pz1, v, acc[39]);
  }
  { const T v = Mc[22];
    acc[22] = fma(T(1), v, acc[22]);
    acc[37] = fma(px1, v, acc[37]);
    acc[40] = fma(py1, v, acc[40]);
    acc[41] = fma(pz1, v, acc[41]);
  }
  { const T v = Mc[23];
    acc[23] = fma(T(1), v, acc[23]);
    acc[38] = fma(px1, v, acc[38]);
    acc[41] = fma(py1, v, acc[41]);
    acc[42] = fma(pz1, v, acc[42]);
  }
  { const T v = Mc[24];
    acc[24] = fma(T(1), v, acc[24]);
    acc[39] = fma(px1, v, acc[39]);
    acc[42] = fma(py1, v, acc[42]);
    acc[43] = fma(pz1, v, acc[43]);
  }
  { const T v = Mc[25];
    acc[25] = fma(T(1), v, acc[25]);
    acc[40] = fma(px1, v, acc[40]);
    acc[44] = fma(py1, v, acc[44]);
    acc[45] = fma(pz1, v, acc[45]);
  }
  { const T v = Mc[26];
    acc[26] = fma(T(1), v, acc[26]);
    acc[41] = fma(px1, v, acc[41]);
    acc[45] = fma(py1, v, acc[45]);
    acc[46] = fma(pz1, v, acc[46]);
  }
  { const T v = Mc[27];
    acc[27] = fma(T(1), v, acc[27]);
    acc[42] = fma(px1, v, acc[42]);
    acc[46] = fma(py1, v, acc[46]);
    acc[47] = fma(pz1, v, acc[47]);
  }
  { const T v = Mc[28];
    acc[28] = fma(T(1), v, acc[28]);
    acc[43] = fma(px1, v, acc[43]);
    acc[47] = fma(py1, v, acc[47]);
    acc[48] = fma(pz1, v, acc[48]);
  }
  { const T v = Mc[29];
    acc[29] = fma(T(1), v, acc[29]);
    acc[44] = fma(px1, v, acc[44]);
    acc[49] = fma(py1, v, acc[49]);
    acc[50] = fma(pz1, v, acc[50]);
  }
  { const T v = Mc[30];
    acc[30] = fma(T(1), v, acc[30]);
    acc[45] = fma(px1, v, acc[45]);
    acc[50] = fma(py1, v, acc[50]);
    acc[51] = fma(pz1, v, acc[51]);
  }
  { const T v = Mc[31];
    acc[31] = fma(T(1), v, acc[31]);
    acc[46] = fma(px1, v, acc[46]);
    acc[51] = fma(py1, v, acc[51]);
    acc[52] = fma(pz1, v, acc[52]);
  }
  { const T v = Mc[32];
    acc[32] = fma(T(1), v, acc[32]);
    acc[47] = fma(px1, v, acc[47]);
    acc[52] = fma(py1, v, acc[52]);
    acc[53] = fma(pz1, v, acc[53]);
  }
  { const T v = Mc[33];
    acc[33] = fma(T(1), v, acc[33]);
    acc[48] = fma(px1, v, acc[48]);
    acc[53] = fma(py1, v, acc[53]);
    acc[54] = fma(pz1, v, acc[54]);
  }
  { const T v = Mc[34];
    acc[34] = fma(T(1), v, acc[34]);
  }
  { const T v = Mc[35];
    acc[35] = fma(T(1), v, acc[35]);
  }
  { const T v = Mc[36];
    acc[36] = fma(T(1), v, acc[36]);
  }
  { const T v = Mc[37];
    acc[37] = fma(T(1), v, acc[37]);
  }
  { const T v = Mc[38];
    acc[38] = fma(T(1), v, acc[38]);
  }
  { const T v = Mc[39];
    acc[39] = fma(T(1), v, acc[39]);
  }
  { const T v = Mc[40];
    acc[40] = fma(T(1), v, acc[40]);
  }
  { const T v = Mc[41];
    acc[41] = fma(T(1), v, acc[41]);
  }
  { const T v = Mc[42];
    acc[42] = fma(T(1), v, acc[42]);
  }
  { const T v = Mc[43];
    acc[43] = fma(T(1), v, acc[43]);
  }
  { const T v = Mc[44];
    acc[44] = fma(T(1), v, acc[44]);
  }
  { const T v = Mc[45];
    acc[45] = fma(T(1), v, acc[45]);
  }
  { const T v = Mc[46];
    acc[46] = fma(T(1), v, acc[46]);
  }
  { const T v = Mc[47];
    acc[47] = fma(T(1), v, acc[47]);
  }
  { const T v = Mc[48];
    acc[48] = fma(T(1), v, acc[48]);
  }
  { const T v = Mc[49];
    acc[49] = fma(T(1), v, acc[49]);
  }
  { const T v = Mc[50];
    acc[50] = fma(T(1), v, acc[50]);
  }
  { const T v = Mc[51];
    acc[51] = fma(T(1), v, acc[51]);
  }
  { const T v = Mc[52];
    acc[52] = fma(T(1), v, acc[52]);
  }
  { const T v = Mc[53];
    acc[53] = fma(T(1), v, acc[53]);
  }
  { const T v = Mc[54];
    acc[54] = fma(T(1), v, acc[54]);
  }
}
// L2L: local expansion Lc about a centre at -(x, y, z) from this one, order 5
template <typename T>
__device__ __forceinline__ void l2l_m1_p5(T x, T y, T z, const T* __restrict__ Lc, T* __restrict__ acc) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  { const T v = Lc[0];
    acc[0] = fma(T(1), v, acc[0]);
  }
  { const T v = Lc[1];
    acc[0] = fma(px1, v, acc[0]);
    acc[1] = fma(T(1), v, acc[1]);
  }
  { const T v = Lc[2];
    acc[0] = fma(py1, v, acc[0]);
    acc[2] = fma(T(1), v, acc[2]);
  }
  { const T v = Lc[3];
    acc[0] = fma(pz1, v, acc[0]);
    acc[3] = fma(T(1), v, acc[3]);
  }
  { const T v = Lc[4];
    acc[0] = fma(px2, v, acc[0]);
    acc[1] = fma(px1, v, acc[1]);
    acc[4] = fma(T(1), v, acc[4]);
  }
  { const T v = Lc[5];
    acc[0] = fma(m_1_1_0, v, acc[0]);
    acc[1] = fma(py1, v, acc[1]);
    acc[2] = fma(px1, v, acc[2]);
    acc[5] = fma(T(1), v, acc[5]);
  }
  { const T v = Lc[6];
    acc[0] = fma(m_1_0_1, v, acc[0]);
    acc[1] = fma(pz1, v, acc[1]);
    acc[3] = fma(px1, v, acc[3]);
    acc[6] = fma(T(1), v, acc[6]);
  }
  { const T v = Lc[7];
    acc[0] = fma(py2, v, acc[0]);
    acc[2] = fma(py1, v, acc[2]);
    acc[7] = fma(T(1), v, acc[7]);
  }
  { const T v = Lc[8];
    acc[0] = fma(m_0_1_1, v, acc[0]);
    acc[2] = fma(pz1, v, acc[2]);
    acc[3] = fma(py1, v, acc[3]);
    acc[8] = fma(T(1), v, acc[8]);
  }
  { const T v = Lc[9];
    acc[0] = fma(pz2, v, acc[0]);
    acc[3] = fma(pz1, v, acc[3]);
    acc[9] = fma(T(1), v, acc[9]);
  }
  { const T v = Lc[10];
    acc[0] = fma(px3, v, acc[0]);
    acc[1] = fma(px2, v, acc[1]);
    acc[4] = fma(px1, v, acc[4]);
    acc[10] = fma(T(1), v, acc[10]);
  }
  { const T v = Lc[11];
    acc[0] = fma(m_2_1_0, v, acc[0]);
    acc[1] = fma(m_1_1_0, v, acc[1]);
    acc[2] = fma(px2, v, acc[2]);
    acc[4] = fma(py1, v, acc[4]);
    acc[5] = fma(px1, v, acc[5]);
    acc[11] = fma(T(1), v, acc[11]);
  }
  { const T v = Lc[12];
    acc[0] = fma(m_2_0_1, v, acc[0]);
    acc[1] = fma(m_1_0_1, v, acc[1]);
    acc[3] = fma(px2, v, acc[3]);
    acc[4] = fma(pz1, v, acc[4]);
    acc[6] = fma(px1, v, acc[6]);
    acc[12] = fma(T(1), v, acc[12]);
  }
  { const T v = Lc[13];
    acc[0] = fma(m_1_2_0, v, acc[0]);
    acc[1] = fma(py2, v, acc[1]);
    acc[2] = fma(m_1_1_0, v, acc[2]);
    acc[5] = fma(py1, v, acc[5]);
    acc[7] = fma(px1, v, acc[7]);
    acc[13] = fma(T(1), v, acc[13]);
  }
  { const T v = Lc[14];
    acc[0] = fma(m_1_1_1, v, acc[0]);
    acc[1] = fma(m_0_1_1, v, acc[1]);
    acc[2] = fma(m_1_0_1, v, acc[2]);
    acc[3] = fma(m_1_1_0, v, acc[3]);
    acc[5] = fma(pz1, v, acc[5]);
    acc[6] = fma(py1, v, acc[6]);
    acc[8] = fma(px1, v, acc[8]);
    acc[14] = fma(T(1), v, acc[14]);
  }
  { const T v = Lc[15];
    acc[0] = fma(m_1_0_2, v, acc[0]);
    acc[1] = fma(pz2, v, acc[1]);
    acc[3] = fma(m_1_0_1, v, acc[3]);
    acc[6] = fma(pz1, v, acc[6]);
    acc[9] = fma(px1, v, acc[9]);
    acc[15] = fma(T(1), v, acc[15]);
  }
  { const T v = Lc[16];
    acc[0] = fma(py3, v, acc[0]);
    acc[2] = fma(py2, v, acc[2]);
    acc[7] = fma(py1, v, acc[7]);
    acc[16] = fma(T(1), v, acc[16]);
  }
  { const T v = Lc[17];
    acc[0] = fma(m_0_2_1, v, acc[0]);
    acc[2] = fma(m_0_1_1, v, acc[2]);
    acc[3] = fma(py2, v, acc[3]);
    acc[7] = fma(pz1, v, acc[7]);
    acc[8] = fma(py1, v, acc[8]);
    acc[17] = fma(T(1), v, acc[17]);
  }
  { const T v = Lc[18];
    acc[0] = fma(m_0_1_2, v, acc[0]);
    acc[2] = fma(pz2, v, acc[2]);
    acc[3] = fma(m_0_1_1, v, acc[3]);
    acc[8] = fma(pz1, v, acc[8]);
    acc[9] = fma(py1, v, acc[9]);
    acc[18] = fma(T(1), v, acc[18]);
  }
  { const T v = Lc[19];
    acc[0] = fma(pz3, v, acc[0]);
    acc[3] = fma(pz2, v, acc[3]);
    acc[9] = fma(pz1, v, acc[9]);
    acc[19] = fma(T(1), v, acc[19]);
  }
  { const T v = Lc[20];
    acc[0] = fma(px4, v, acc[0]);
    acc[1] = fma(px3, v, acc[1]);
    acc[4] = fma(px2, v, acc[4]);
    acc[10] = fma(px1, v, acc[10]);
    acc[20] = fma(T(1), v, acc[20]);
  }
  { const T v = Lc[21];
    acc[0] = fma(m_3_1_0, v, acc[0]);
    acc[1] = fma(m_2_1_0, v, acc[1]);
    acc[2] = fma(px3, v, acc[2]);
    acc[4] = fma(m_1_1_0, v, acc[4]);
    acc[5] = fma(px2, v, acc[5]);
    acc[10] = fma(py1, v, acc[10]);
    acc[11] = fma(px1, v, acc[11]);
    acc[21] = fma(T(1), v, acc[21]);
  }
  { const T v = Lc[22];
    acc[0] = fma(m_3_0_1, v, acc[0]);
    acc[1] = fma(m_2_0_1, v, acc[1]);
    acc[3] = fma(px3, v, acc[3]);
    acc[4] = fma(m_1_0_1, v, acc[4]);
    acc[6] = fma(px2, v, acc[6]);
    acc[10] = fma(pz1, v, acc[10]);
    acc[12] = fma(px1, v, acc[12]);
    acc[22] = fma(T(1), v, acc[22]);
  }
  { const T v = Lc[23];
    acc[0] = fma(m_2_2_0, v, acc[0]);
    acc[1] = fma(m_1_2_0, v, acc[1]);
    acc[2] = fma(m_2_1_0, v, acc[2]);
    acc[4] = fma(py2, v, acc[4]);
    acc[5] = fma(m_1_1_0, v, acc[5]);
    acc[7] = fma(px2, v, acc[7]);
    acc[11] = fma(py1, v, acc[11]);
    acc[13] = fma(px1, v, acc[13]);
    acc[23] = fma(T(1), v, acc[23]);
  }
  { const T v = Lc[24];
    acc[0] = fma(m_2_1_1, v, acc[0]);
    acc[1] = fma(m_1_1_1, v, acc[1]);
    acc[2] = fma(m_2_0_1, v, acc[2]);
    acc[3] = fma(m_2_1_0, v, acc[3]);
    acc[4] = fma(m_0_1_1, v, acc[4]);
    acc[5] = fma(m_1_0_1, v, acc[5]);
    acc[6] = fma(m_1_1_0, v, acc[6]);
    acc[8] = fma(px2, v, acc[8]);
    acc[11] = fma(pz1, v, acc[11]);
    acc[12] = fma(py1, v, acc[12]);
    acc[14] = fma(px1, v, acc[14]);
    acc[24] = fma(T(1), v, acc[24]);
  }
  { const T v = Lc[25];
    acc[0] = fma(m_2_0_2, v, acc[0]);
    acc[1] = fma(m_1_0_2, v, acc[1]);
    acc[3] = fma(m_2_0_1, v, acc[3]);
    acc[4] = fma(pz2, v, acc[4]);
    acc[6] = fma(m_1_0_1, v, acc[6]);
    acc[9] = fma(px2, v, acc[9]);
    acc[12] = fma(pz1, v, acc[12]);
    acc[15] = fma(px1, v, acc[15]);
    acc[25] = fma(T(1), v, acc[25]);
  }
  { const T v = Lc[26];
    acc[0] = fma(m_1_3_0, v, acc[0]);
    acc[1] = fma(py3, v, acc[1]);
    acc[2] = fma(m_1_2_0, v, acc[2]);
    acc[5] = fma(py2, v, acc[5]);
    acc[7] = fma(m_1_1_0, v, acc[7]);
    acc[13] = fma(py1, v, acc[13]);
    acc[16] = fma(px1, v, acc[16]);
    acc[26] = fma(T(1), v, acc[26]);
  }
  { const T v = Lc[27];
    acc[0] = fma(m_1_2_1, v, acc[0]);
    acc[1] = fma(m_0_2_1, v, acc[1]);
    acc[2] = fma(m_1_1_1, v, acc[2]);
    acc[3] = fma(m_1_2_0, v, acc[3]);
    acc[5] = fma(m_0_1_1, v, acc[5]);
    acc[6] = fma(py2, v, acc[6]);
    acc[7] = fma(m_1_0_1, v, acc[7]);
    acc[8] = fma(m_1_1_0, v, acc[8]);
    acc[13] = fma(pz1, v, acc[13]);
    acc[14] = fma(py1, v, acc[14]);
    acc[17] = fma(px1, v, acc[17]);
    acc[27] = fma(T(1), v, acc[27]);
  }
  { const T v = Lc[28];
    acc[0] = fma(m_1_1_2, v, acc[0]);
    acc[1] = fma(m_0_1_2, v, acc[1]);
    acc[2] = fma(m_1_0_2, v, acc[2]);
    acc[3] = fma(m_1_1_1, v, acc[3]);
    acc[5] = fma(pz2, v, acc[5]);
    acc[6] = fma(m_0_1_1, v, acc[6]);
    acc[8] = fma(m_1_0_1, v, acc[8]);
    acc[9] = fma(m_1_1_0, v, acc[9]);
    acc[14] = fma(pz1, v, acc[14]);
    acc[15] = fma(py1, v, acc[15]);
    acc[18] = fma(px1, v, acc[18]);
    acc[28] = fma(T(1), v, acc[28]);
  }
  { const T v = Lc[29];
    acc[0] = fma(m_1_0_3, v, acc[0]);
    acc[1] = fma(pz3, v, acc[1]);
    acc[3] = fma(m_1_0_2, v, acc[3]);
    acc[6] = fma(pz2, v, acc[6]);
    acc[9] = fma(m_1_0_1, v, acc[9]);
    acc[15] = fma(pz1, v, acc[15]);
    acc[19] = fma(px1, v, acc[19]);
    acc[29] = fma(T(1), v, acc[29]);
  }
  { const T v = Lc[30];
    acc[0] = fma(py4, v, acc[0]);
    acc[2] = fma(py3, v, acc[2]);
    acc[7] = fma(py2, v, acc[7]);
    acc[16] = fma(py1, v, acc[16]);
    acc[30] = fma(T(1), v, acc[30]);
  }
  { const T v = Lc[31];
    acc[0] = fma(m_0_3_1, v, acc[0]);
    acc[2] = fma(m_0_2_1, v, acc[2]);
    acc[3] = fma(py3, v, acc[3]);
    acc[7] = fma(m_0_1_1, v, acc[7]);
    acc[8] = fma(py2, v, acc[8]);
    acc[16] = fma(pz1, v, acc[16]);
    acc[17] = fma(py1, v, acc[17]);
    acc[31] = fma(T(1), v, acc[31]);
  }
  { const T v = Lc[32];
    acc[0] = fma(m_0_2_2, v, acc[0]);
    acc[2] = fma(m_0_1_2, v, acc[2]);
    acc[3] = fma(m_0_2_1, v, acc[3]);
    acc[7] = fma(pz2, v, acc[7]);
    acc[8] = fma(m_0_1_1, v, acc[8]);
    acc[9] = fma(py2, v, acc[9]);
    acc[17] = fma(pz1, v, acc[17]);
    acc[18] = fma(py1, v, acc[18]);
    acc[32] = fma(T(1), v, acc[32]);
  }
  { const T v = Lc[33];
    acc[0] = fma(m_0_1_3, v, acc[0]);
    acc[2] = fma(pz3, v, acc[2]);
    acc[3] = fma(m_0_1_2, v, acc[3]);
    acc[8] = fma(pz2, v, acc[8]);
    acc[9] = fma(m_0_1_1, v, acc[9]);
    acc[18] = fma(pz1, v, acc[18]);
    acc[19] = fma(py1, v, acc[19]);
    acc[33] = fma(T(1), v, acc[33]);
  }
  { const T v = Lc[34];
    acc[0] = fma(pz4, v, acc[0]);
    acc[3] = fma(pz3, v, acc[3]);
    acc[9] = fma(pz2, v, acc[9]);
    acc[19] = fma(pz1, v, acc[19]);
    acc[34] = fma(T(1), v, acc[34]);
  }
}
// L2P: field -grad of the local expansion Lc at offset (x, y, z) = site - centre, order 5
template <typename T>
__device__ __forceinline__ void l2p_m1_p5(T x, T y, T z, const T* __restrict__ Lc, T& f0, T& f1, T& f2) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  { const T v = -Lc[1];
    f0 = fma(T(1), v, f0);
  }
  { const T v = -Lc[2];
    f1 = fma(T(1), v, f1);
  }
  { const T v = -Lc[3];
    f2 = fma(T(1), v, f2);
  }
  { const T v = -Lc[4];
    f0 = fma(px1, v, f0);
  }
  { const T v = -Lc[5];
    f0 = fma(py1, v, f0);
    f1 = fma(px1, v, f1);
  }
  { const T v = -Lc[6];
    f0 = fma(pz1, v, f0);
    f2 = fma(px1, v, f2);
  }
  { const T v = -Lc[7];
    f1 = fma(py1, v, f1);
  }
  { const T v = -Lc[8];
    f1 = fma(pz1, v, f1);
    f2 = fma(py1, v, f2);
  }
  { const T v = -Lc[9];
    f2 = fma(pz1, v, f2);
  }
  { const T v = -Lc[10];
    f0 = fma(px2, v, f0);
  }
  { const T v = -Lc[11];
    f0 = fma(m_1_1_0, v, f0);
    f1 = fma(px2, v, f1);
  }
  { const T v = -Lc[12];
    f0 = fma(m_1_0_1, v, f0);
    f2 = fma(px2, v, f2);
  }
  { const T v = -Lc[13];
    f0 = fma(py2, v, f0);
    f1 = fma(m_1_1_0, v, f1);
  }
  { const T v = -Lc[14];
    f0 = fma(m_0_1_1, v, f0);
    f1 = fma(m_1_0_1, v, f1);
    f2 = fma(m_1_1_0, v, f2);
  }
  { const T v = -Lc[15];
    f0 = fma(pz2, v, f0);
    f2 = fma(m_1_0_1, v, f2);
  }
  { const T v = -Lc[16];
    f1 = fma(py2, v, f1);
  }
  { const T v = -Lc[17];
    f1 = fma(m_0_1_1, v, f1);
    f2 = fma(py2, v, f2);
  }
  { const T v = -Lc[18];
    f1 = fma(pz2, v, f1);
    f2 = fma(m_0_1_1, v, f2);
  }
  { const T v = -Lc[19];
    f2 = fma(pz2, v, f2);
  }
  { const T v = -Lc[20];
    f0 = fma(px3, v, f0);
  }
  { const T v = -Lc[21];
    f0 = fma(m_2_1_0, v, f0);
    f1 = fma(px3, v, f1);
  }
  { const T v = -Lc[22];
    f0 = fma(m_2_0_1, v, f0);
    f2 = fma(px3, v, f2);
  }
  { const T v = -Lc[23];
    f0 = fma(m_1_2_0, v, f0);
    f1 = fma(m_2_1_0, v, f1);
  }
  { const T v = -Lc[24];
    f0 = fma(m_1_1_1, v, f0);
    f1 = fma(m_2_0_1, v, f1);
    f2 = fma(m_2_1_0, v, f2);
  }
  { const T v = -Lc[25];
    f0 = fma(m_1_0_2, v, f0);
    f2 = fma(m_2_0_1, v, f2);
  }
  { const T v = -Lc[26];
    f0 = fma(py3, v, f0);
    f1 = fma(m_1_2_0, v, f1);
  }
  { const T v = -Lc[27];
    f0 = fma(m_0_2_1, v, f0);
    f1 = fma(m_1_1_1, v, f1);
    f2 = fma(m_1_2_0, v, f2);
  }
  { const T v = -Lc[28];
    f0 = fma(m_0_1_2, v, f0);
    f1 = fma(m_1_0_2, v, f1);
    f2 = fma(m_1_1_1, v, f2);
  }
  { const T v = -Lc[29];
    f0 = fma(pz3, v, f0);
    f2 = fma(m_1_0_2, v, f2);
  }
  { const T v = -Lc[30];
    f1 = fma(py3, v, f1);
  }
  { const T v = -Lc[31];
    f1 = fma(m_0_2_1, v, f1);
    f2 = fma(py3, v, f2);
  }
  { const T v = -Lc[32];
    f1 = fma(m_0_1_2, v, f1);
    f2 = fma(m_0_2_1, v, f2);
  }
  { const T v = -Lc[33];
    f1 = fma(pz3, v, f1);
    f2 = fma(m_0_1_2, v, f2);
  }
  { const T v = -Lc[34];
    f2 = fma(pz3, v, f2);
  }
}

// P2M of a dipole (s0, s1, s2) at offset (x, y, z) = centre - site, order 6
template <typename T>
__device__ __forceinline__ void p2m_m1_p6(T x, T y, T z, T s0, T s1, T s2, T* __restrict__ acc) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T px5 = px4 * x * cinv<T>(5);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T py5 = py4 * y * cinv<T>(5);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T pz5 = pz4 * z * cinv<T>(5);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  const T m_4_1_0 = px4 * py1;
  const T m_4_0_1 = px4 * pz1;
  const T m_3_2_0 = px3 * py2;
  const T m_3_1_1 = px3 * py1 * pz1;
  const T m_3_0_2 = px3 * pz2;
  const T m_2_3_0 = px2 * py3;
  const T m_2_2_1 = px2 * py2 * pz1;
  const T m_2_1_2 = px2 * py1 * pz2;
  const T m_2_0_3 = px2 * pz3;
  const T m_1_4_0 = px1 * py4;
  const T m_1_3_1 = px1 * py3 * pz1;
  const T m_1_2_2 = px1 * py2 * pz2;
  const T m_1_1_3 = px1 * py1 * pz3;
  const T m_1_0_4 = px1 * pz4;
  const T m_0_4_1 = py4 * pz1;
  const T m_0_3_2 = py3 * pz2;
  const T m_0_2_3 = py2 * pz3;
  const T m_0_1_4 = py1 * pz4;
  { const T v = s0;
    acc[0] = fma(T(1), v, acc[0]);
    acc[3] = fma(px1, v, acc[3]);
    acc[4] = fma(py1, v, acc[4]);
    acc[5] = fma(pz1, v, acc[5]);
    acc[9] = fma(px2, v, acc[9]);
    acc[10] = fma(m_1_1_0, v, acc[10]);
    acc[11] = fma(m_1_0_1, v, acc[11]);
    acc[12] = fma(py2, v, acc[12]);
    acc[13] = fma(m_0_1_1, v, acc[13]);
    acc[14] = fma(pz2, v, acc[14]);
    acc[19] = fma(px3, v, acc[19]);
    acc[20] = fma(m_2_1_0, v, acc[20]);
    acc[21] = fma(m_2_0_1, v, acc[21]);
    acc[22] = fma(m_1_2_0, v, acc[22]);
    acc[23] = fma(m_1_1_1, v, acc[23]);
    acc[24] = fma(m_1_0_2, v, acc[24]);
    acc[25] = fma(py3, v, acc[25]);
    acc[26] = fma(m_0_2_1, v, acc[26]);
    acc[27] = fma(m_0_1_2, v, acc[27]);
    acc[28] = fma(pz3, v, acc[28]);
    acc[34] = fma(px4, v, acc[34]);
    acc[35] = fma(m_3_1_0, v, acc[35]);
    acc[36] = fma(m_3_0_1, v, acc[36]);
    acc[37] = fma(m_2_2_0, v, acc[37]);
    acc[38] = fma(m_2_1_1, v, acc[38]);
    acc[39] = fma(m_2_0_2, v, acc[39]);
    acc[40] = fma(m_1_3_0, v, acc[40]);
    acc[41] = fma(m_1_2_1, v, acc[41]);
    acc[42] = fma(m_1_1_2, v, acc[42]);
    acc[43] = fma(m_1_0_3, v, acc[43]);
    acc[44] = fma(py4, v, acc[44]);
    acc[45] = fma(m_0_3_1, v, acc[45]);
    acc[46] = fma(m_0_2_2, v, acc[46]);
    acc[47] = fma(m_0_1_3, v, acc[47]);
    acc[48] = fma(pz4, v, acc[48]);
    acc[55] = fma(px5, v, acc[55]);
    acc[56] = fma(m_4_1_0, v, acc[56]);
    acc[57] = fma(m_4_0_1, v, acc[57]);
    acc[58] = fma(m_3_2_0, v, acc[58]);
    acc[59] = fma(m_3_1_1, v, acc[59]);
    acc[60] = fma(m_3_0_2, v, acc[60]);
    acc[61] = fma(m_2_3_0, v, acc[61]);
    acc[62] = fma(m_2_2_1, v, acc[62]);
    acc[63] = fma(m_2_1_2, v, acc[63]);
    acc[64] = fma(m_2_0_3, v, acc[64]);
    acc[65] = fma(m_1_4_0, v, acc[65]);
    acc[66] = fma(m_1_3_1, v, acc[66]);
    acc[67] = fma(m_1_2_2, v, acc[67]);
    acc[68] = fma(m_1_1_3, v, acc[68]);
    acc[69] = fma(m_1_0_4, v, acc[69]);
    acc[70] = fma(py5, v, acc[70]);
    acc[71] = fma(m_0_4_1, v, acc[71]);
    acc[72] = fma(m_0_3_2, v, acc[72]);
    acc[73] = fma(m_0_2_3, v, acc[73]);
    acc[74] = fma(m_0_1_4, v, acc[74]);
    acc[75] = fma(pz5, v, acc[75]);
  }
  { const T v = s1;
    acc[1] = fma(T(1), v, acc[1]);
    acc[4] = fma(px1, v, acc[4]);
    acc[6] = fma(py1, v, acc[6]);
    acc[7] = fma(pz1, v, acc[7]);
    acc[10] = fma(px2, v, acc[10]);
    acc[12] = fma(m_1_1_0, v, acc[12]);
    acc[13] = fma(m_1_0_1, v, acc[13]);
    acc[15] = fma(py2, v, acc[15]);
    acc[16] = fma(m_0_1_1, v, acc[16]);
    acc[17] = fma(pz2, v, acc[17]);
    acc[20] = fma(px3, v, acc[20]);
    acc[22] = fma(m_2_1_0, v, acc[22]);
    acc[23] = fma(m_2_0_1, v, acc[23]);
    acc[25] = fma(m_1_2_0, v, acc[25]);
    acc[26] = fma(m_1_1_1, v, acc[26]);
    acc[27] = fma(m_1_0_2, v, acc[27]);
    acc[29] = fma(py3, v, acc[29]);
    acc[30] = fma(m_0_2_1, v, acc[30]);
    acc[31] = fma(m_0_1_2, v, acc[31]);
    acc[32] = fma(pz3, v, acc[32]);
    acc[35] = fma(px4, v, acc[35]);
    acc[37] = fma(m_3_1_0, v, acc[37]);
    acc[38] = fma(m_3_0_1, v, acc[38]);
    acc[40] = fma(m_2_2_0, v, acc[40]);
    acc[41] = fma(m_2_1_1, v, acc[41]);
    acc[42] = fma(m_2_0_2, v, acc[42]);
    acc[44] = fma(m_1_3_0, v, acc[44]);
    acc[45] = fma(m_1_2_1, v, acc[45]);
    acc[46] = fma(m_1_1_2, v, acc[46]);
    acc[47] = fma(m_1_0_3, v, acc[47]);
    acc[49] = fma(py4, v, acc[49]);
    acc[50] = fma(m_0_3_1, v, acc[50]);
    acc[51] = fma(m_0_2_2, v, acc[51]);
    acc[52] = fma(m_0_1_3, v, acc[52]);
    acc[53] = fma(pz4, v, acc[53]);
    acc[56] = fma(px5, v, acc[56]);
    acc[58] = fma(m_4_1_0, v, acc[58]);
    acc[59] = fma(m_4_0_1, v, acc[59]);
    acc[61] = fma(m_3_2_0, v, acc[61]);
    acc[62] = fma(m_3_1_1, v, acc[62]);
    acc[63] = fma(m_3_0_2, v, acc[63]);
    acc[65] = fma(m_2_3_0, v, acc[65]);
    acc[66] = fma(m_2_2_1, v, acc[66]);
    acc[67] = fma(m_2_1_2, v, acc[67]);
    acc[68] = fma(m_2_0_3, v, acc[68]);
    acc[70] = fma(m_1_4_0, v, acc[70]);
    acc[71] = fma(m_1_3_1, v, acc[71]);
    acc[72] = fma(m_1_2_2, v, acc[72]);
    acc[73] = fma(m_1_1_3, v, acc[73]);
    acc[74] = fma(m_1_0_4, v, acc[74]);
    acc[76] = fma(py5, v, acc[76]);
    acc[77] = fma(m_0_4_1, v, acc[77]);
    acc[78] = fma(m_0_3_2, v, acc[78]);
    acc[79] = fma(m_0_2_3, v, acc[79]);
    acc[80] = fma(m_0_1_4, v, acc[80]);
    acc[81] = fma(pz5, v, acc[81]);
  }
  { const T v = s2;
    acc[2] = fma(T(1), v, acc[2]);
    acc[5] = fma(px1, v, acc[5]);
    acc[7] = fma(py1, v, acc[7]);
    acc[8] = fma(pz1, v, acc[8]);
    acc[11] = fma(px2, v, acc[11]);
    acc[13] = fma(m_1_1_0, v, acc[13]);
    acc[14] = fma(m_1_0_1, v, acc[14]);
    acc[16] = fma(py2, v, acc[16]);
    acc[17] = fma(m_0_1_1, v, acc[17]);
    acc[18] = fma(pz2, v, acc[18]);
    acc[21] = fma(px3, v, acc[21]);
    acc[23] = fma(m_2_1_0, v, acc[23]);
    acc[24] = fma(m_2_0_1, v, acc[24]);
    acc[26] = fma(m_1_2_0, v, acc[26]);
    acc[27] = fma(m_1_1_1, v, acc[27]);
    acc[28] = fma(m_1_0_2, v, acc[28]);
    acc[30] = fma(py3, v, acc[30]);
    acc[31] = fma(m_0_2_1, v, acc[31]);
    acc[32] = fma(m_0_1_2, v, acc[32]);
    acc[33] = fma(pz3, v, acc[33]);
    acc[36] = fma(px4, v, acc[36]);
    acc[38] = fma(m_3_1_0, v, acc[38]);
    acc[39] = fma(m_3_0_1, v, acc[39]);
    acc[41] = fma(m_2_2_0, v, acc[41]);
    acc[42] = fma(m_2_1_1, v, acc[42]);
    acc[43] = fma(m_2_0_2, v, acc[43]);
    acc[45] = fma(m_1_3_0, v, acc[45]);
    acc[46] = fma(m_1_2_1, v, acc[46]);
    acc[47] = fma(m_1_1_2, v, acc[47]);
    acc[48] = fma(m_1_0_3, v, acc[48]);
    acc[50] = fma(py4, v, acc[50]);
    acc[51] = fma(m_0_3_1, v, acc[51]);
    acc[52] = fma(m_0_2_2, v, acc[52]);
    acc[53] = fma(m_0_1_3, v, acc[53]);
    acc[54] = fma(pz4, v, acc[54]);
    acc[57] = fma(px5, v, acc[57]);
    acc[59] = fma(m_4_1_0, v, acc[59]);
    acc[60] = fma(m_4_0_1, v, acc[60]);
    acc[62] = fma(m_3_2_0, v, acc[62]);
    acc[63] = fma(m_3_1_1, v, acc[63]);
    acc[64] = fma(m_3_0_2, v, acc[64]);
    acc[66] = fma(m_2_3_0, v, acc[66]);
    acc[67] = fma(m_2_2_1, v, acc[67]);
    acc[68] = fma(m_2_1_2, v, acc[68]);
    acc[69] = fma(m_2_0_3, v, acc[69]);
    acc[71] = fma(m_1_4_0, v, acc[71]);
    acc[72] = fma(m_1_3_1, v, acc[72]);
    acc[73] = fma(m_1_2_2, v, acc[73]);
    acc[74] = fma(m_1_1_3, v, acc[74]);
    acc[75] = fma(m_1_0_4, v, acc[75]);
    acc[77] = fma(py5, v, acc[77]);
    acc[78] = fma(m_0_4_1, v, acc[78]);
    acc[79] = fma(m_0_3_2, v, acc[79]);
    acc[80] = fma(m_0_2_3, v, acc[80]);
    acc[81] = fma(m_0_1_4, v, acc[81]);
    acc[82] = fma(pz5, v, acc[82]);
  }
}
// M2M: multipole Mc about a centre at (x, y, z) from this one, order 6
template <typename T>
__device__ __forceinline__ void m2m_m1_p6(T x, T y, T z, const T* __restrict__ Mc, T* __restrict__ acc) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T px5 = px4 * x * cinv<T>(5);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T py5 = py4 * y * cinv<T>(5);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T pz5 = pz4 * z * cinv<T>(5);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  const T m_4_1_0 = px4 * py1;
  const T m_4_0_1 = px4 * pz1;
  const T m_3_2_0 = px3 * py2;
  const T m_3_1_1 = px3 * py1 * pz1;
  const T m_3_0_2 = px3 * pz2;
  const T m_2_3_0 = px2 * py3;
  const T m_2_2_1 = px2 * py2 * pz1;
  const T m_2_1_2 = px2 * py1 * pz2;
  const T m_2_0_3 = px2 * pz3;
  const T m_1_4_0 = px1 * py4;
  const T m_1_3_1 = px1 * py3 * pz1;
  const T m_1_2_2 = px1 * py2 * pz2;
  const T m_1_1_3 = px1 * py1 * pz3;
  const T m_1_0_4 = px1 * pz4;
  const T m_0_4_1 = py4 * pz1;
  const T m_0_3_2 = py3 * pz2;
  const T m_0_2_3 = py2 * pz3;
  const T m_0_1_4 = py1 * pz4;
  { const T v = Mc[0];
    acc[0] = fma(T(1), v, acc[0]);
    acc[3] = fma(px1, v, acc[3]);
    acc[4] = fma(py1, v, acc[4]);
    acc[5] = fma(pz1, v, acc[5]);
    acc[9] = fma(px2, v, acc[9]);
    acc[10] = fma(m_1_1_0, v, acc[10]);
    acc[11] = fma(m_1_0_1, v, acc[11]);
    acc[12] = fma(py2, v, acc[12]);
    acc[13] = fma(m_0_1_1, v, acc[13]);
    acc[14] = fma(pz2, v, acc[14]);
    acc[19] = fma(px3, v, acc[19]);
    acc[20] = fma(m_2_1_0, v, acc[20]);
    acc[21] = fma(m_2_0_1, v, acc[21]);
    acc[22] = fma(m_1_2_0, v, acc[22]);
    acc[23] = fma(m_1_1_1, v, acc[23]);
    acc[24] = fma(m_1_0_2, v, acc[24]);
    acc[25] = fma(py3, v, acc[25]);
    acc[26] = fma(m_0_2_1, v, acc[26]);
    acc[27] = fma(m_0_1_2, v, acc[27]);
    acc[28] = fma(pz3, v, acc[28]);
    acc[34] = fma(px4, v, acc[34]);
    acc[35] = fma(m_3_1_0, v, acc[35]);
    acc[36] = fma(m_3_0_1, v, acc[36]);
    acc[37] = fma(m_2_2_0, v, acc[37]);
    acc[38] = fma(m_2_1_1, v, acc[38]);
    acc[39] = fma(m_2_0_2, v, acc[39]);
    acc[40] = fma(m_1_3_0, v, acc[40]);
    acc[41] = fma(m_1_2_1, v, acc[41]);
    acc[42] = fma(m_1_1_2, v, acc[42]);
    acc[43] = fma(m_1_0_3, v, acc[43]);
    acc[44] = fma(py4, v, acc[44]);
    acc[45] = fma(m_0_3_1, v, acc[45]);
    acc[46] = fma(m_0_2_2, v, acc[46]);
    acc[47] = fma(m_0_1_3, v, acc[47]);
    acc[48] = fma(pz4, v, acc[48]);
    acc[55] = fma(px5, v, acc[55]);
    acc[56] = fma(m_4_1_0, v, acc[56]);
    acc[57] = fma(m_4_0_1, v, acc[57]);
    acc[58] = fma(m_3_2_0, v, acc[58]);
    acc[59] = fma(m_3_1_1, v, acc[59]);
    acc[60] = fma(m_3_0_2, v, acc[60]);
    acc[61] = fma(m_2_3_0, v, acc[61]);
    acc[62] = fma(m_2_2_1, v, acc[62]);
    acc[63] = fma(m_2_1_2, v, acc[63]);
    acc[64] = fma(m_2_0_3, v, acc[64]);
    acc[65] = fma(m_1_4_0, v, acc[65]);
    acc[66] = fma(m_1_3_1, v, acc[66]);
    acc[67] = fma(m_1_2_2, v, acc[67]);
    acc[68] = fma(m_1_1_3, v, acc[68]);
    acc[69] = fma(m_1_0_4, v, acc[69]);
    acc[70] = fma(py5, v, acc[70]);
    acc[71] = fma(m_0_4_1, v, acc[71]);
    acc[72] = fma(m_0_3_2, v, acc[72]);
    acc[73] = fma(m_0_2_3, v, acc[73]);
    acc[74] = fma(m_0_1_4, v, acc[74]);
    acc[75] = fma(pz5, v, acc[75]);
  }
  { const T v = Mc[1];
    acc[1] = fma(T(1), v, acc[1]);
    acc[4] = fma(px1, v, acc[4]);
    acc[6] = fma(py1, v, acc[6]);
    acc[7] = fma(pz1, v, acc[7]);
    acc[10] = fma(px2, v, acc[10]);
    acc[12] = fma(m_1_1_0, v, acc[12]);
    acc[13] = fma(m_1_0_1, v, acc[13]);
    acc[15] = fma(py2, v, acc[15]);
    acc[16] = fma(m_0_1_1, v, acc[16]);
    acc[17] = fma(pz2, v, acc[17]);
    acc[20] = fma(px3, v, acc[20]);
    acc[22] = fma(m_2_1_0, v, acc[22]);
    acc[23] = fma(m_2_0_1, v, acc[23]);
    acc[25] = fma(m_1_2_0, v, acc[25]);
    acc[26] = fma(m_1_1_1, v, acc[26]);
    acc[27] = fma(m_1_0_2, v, acc[27]);
    acc[29] = fma(py3, v, acc[29]);
    acc[30] = fma(m_0_2_1, v, acc[30]);
    acc[31] = fma(m_0_1_2, v, acc[31]);
    acc[32] = fma(pz3, v, acc[32]);
    acc[35] = fma(px4, v, acc[35]);
    acc[37] = fma(m_3_1_0, v, acc[37]);
    acc[38] = fma(m_3_0_1, v, acc[38]);
    acc[40] = fma(m_2_2_0, v, acc[40]);
    acc[41] = fma(m_2_1_1, v, acc[41]);
    acc[42] = fma(m_2_0_2, v, acc[42]);
    acc[44] = fma(m_1_3_0, v, acc[44]);
    acc[45] = fma(m_1_2_1, v, acc[45]);
    acc[46] = fma(m_1_1_2, v, acc[46]);
    acc[47] = fma(m_1_0_3, v, acc[47]);
    acc[49] = fma(py4, v, acc[49]);
    acc[50] = fma(m_0_3_1, v, acc[50]);
    acc[51] = fma(m_0_2_2, v, acc[51]);
    acc[52] = fma(m_0_1_3, v, acc[52]);
    acc[53] = fma(pz4, v, acc[53]);
    acc[56] = fma(px5, v, acc[56]);
    acc[58] = fma(m_4_1_0, v, acc[58]);
    acc[59] = fma(m_4_0_1, v, acc[59]);
    acc[61] = fma(m_3_2_0, v, acc[61]);
    acc[62] = fma(m_3_1_1, v, acc[62]);
    acc[63] = fma(m_3_0_2, v, acc[63]);
    acc[65] = fma(m_2_3_0, v, acc[65]);
    acc[66] = fma(m_2_2_1, v, acc[66]);
    acc[67] = fma(m_2_1_2, v, acc[67]);
    acc[68] = fma(m_2_0_3, v, acc[68]);
    acc[70] = fma(m_1_4_0, v, acc[70]);
    acc[71] = fma(m_1_3_1, v, acc[71]);
    acc[72] = fma(m_1_2_2, v, acc[72]);
    acc[73] = fma(m_1_1_3, v, acc[73]);
    acc[74] = fma(m_1_0_4, v, acc[74]);
    acc[76] = fma(py5, v, acc[76]);
    acc[77] = fma(m_0_4_1, v, acc[77]);
    acc[78] = fma(m_0_3_2, v, acc[78]);
    acc[79] = fma(m_0_2_3, v, acc[79]);
    acc[80] = fma(m_0_1_4, v, acc[80]);
    acc[81] = fma(pz5, v, acc[81]);
  }
  { const T v = Mc[2];
    acc[2] = fma(T(1), v, acc[2]);
    acc[5] = fma(px1, v, acc[5]);
    acc[7] = fma(py1, v, acc[7]);
    acc[8] = fma(pz1, v, acc[8]);
    acc[11] = fma(px2, v, acc[11]);
    acc[13] = fma(m_1_1_0, v, acc[13]);
    acc[14] = fma(m_1_0_1, v, acc[14]);
    acc[16] = fma(py2, v, acc[16]);
    acc[17] = fma(m_0_1_1, v, acc[17]);
    acc[18] = fma(pz2, v, acc[18]);
    acc[21] = fma(px3, v, acc[21]);
    acc[23] = fma(m_2_1_0, v, acc[23]);
    acc[24] = fma(m_2_0_1, v, acc[24]);
    acc[26] = fma(m_1_2_0, v, acc[26]);
    acc[27] = fma(m_1_1_1, v, acc[27]);
    acc[28] = fma(m_1_0_2, v, acc[28]);
    acc[30] = fma(py3, v, acc[30]);
    acc[31] = fma(m_0_2_1, v, acc[31]);
    acc[32] = fma(m_0_1_2, v, acc[32]);
    acc[33] = fma(pz3, v, acc[33]);
    acc[36] = fma(px4, v, acc[36]);
    acc[38] = fma(m_3_1_0, v, acc[38]);
    acc[39] = fma(m_3_0_1, v, acc[39]);
    acc[41] = fma(m_2_2_0, v, acc[41]);
    acc[42] = fma(m_2_1_1, v, acc[42]);
    acc[43] = fma(m_2_0_2, v, acc[43]);
    acc[45] = fma(m_1_3_0, v, acc[45]);
    acc[46] = fma(m_1_2_1, v, acc[46]);
    acc[47] = fma(m_1_1_2, v, acc[47]);
    acc[48] = fma(m_1_0_3, v, acc[48]);
    acc[50] = fma(py4, v, acc[50]);
    acc[51] = fma(m_0_3_1, v, acc[51]);
    acc[52] = fma(m_0_2_2, v, acc[52]);
    acc[53] = fma(m_0_1_3, v, acc[53]);
    acc[54] = fma(pz4, v, acc[54]);
    acc[57] = fma(px5, v, acc[57]);
    acc[59] = fma(m_4_1_0, v, acc[59]);
    acc[60] = fma(m_4_0_1, v, acc[60]);
    acc[62] = fma(m_3_2_0, v, acc[62]);
    acc[63] = fma(m_3_1_1, v, acc[63]);
    acc[64] = fma(m_3_0_2, v, acc[64]);
    acc[66] = fma(m_2_3_0, v, acc[66]);
    acc[67] = fma(m_2_2_1, v, acc[67]);
    acc[68] = fma(m_2_1_2, v, acc[68]);
    acc[69] = fma(m_2_0_3, v, acc[69]);
    acc[71] = fma(m_1_4_0, v, acc[71]);
    acc[72] = fma(m_1_3_1, v, acc[72]);
    acc[73] = fma(m_1_2_2, v, acc[73]);
    acc[74] = fma(m_1_1_3, v, acc[74]);
    acc[75] = fma(m_1_0_4, v, acc[75]);
    acc[77] = fma(py5, v, acc[77]);
    acc[78] = fma(m_0_4_1, v, acc[78]);
    acc[79] = fma(m_0_3_2, v, acc[79]);
    acc[80] = fma(m_0_2_3, v, acc[80]);
    acc[81] = fma(m_0_1_4, v, acc[81]);
    acc[82] = fma(pz5, v, acc[82]);
  }
  { const T v = Mc[3];
    acc[3] = fma(T(1), v, acc[3]);
    acc[9] = fma(px1, v, acc[9]);
    acc[10] = fma(py1, v, acc[10]);
    acc[11] = fma(pz1, v, acc[11]);
    acc[19] = fma(px2, v, acc[19]);
    acc[20] = fma(m_1_1_0, v, acc[20]);
    acc[21] = fma(m_1_0_1, v, acc[21]);
    acc[22] = fma(py2, v, acc[22]);
    acc[23] = fma(m_0_1_1, v, acc[23]);
    acc[24] = fma(pz2, v, acc[24]);
    acc[34] = fma(px3, v, acc[34]);
    acc[35] = fma(m_2_1_0, v, acc[35]);
    acc[36] = fma(m_2_0_1, v, acc[36]);
    acc[37] = fma(m_1_2_0, v, acc[37]);
    acc[38] = fma(m_1_1_1, v, acc[38]);
    acc[39] = fma(m_1_0_2, v, acc[39]);
    acc[40] = fma(py3, v, acc[40]);
    acc[41] = fma(m_0_2_1, v, acc[41]);
    acc[42] = fma(m_0_1_2, v, acc[42]);
    acc[43] = fma(pz3, v, acc[43]);
    acc[55] = fma(px4, v, acc[55]);
    acc[56] = fma(m_3_1_0, v, acc[56]);
    acc[57] = fma(m_3_0_1, v, acc[57]);
    acc[58] = fma(m_2_2_0, v, acc[58]);
    acc[59] = fma(m_2_1_1, v, acc[59]);
    acc[60] = fma(m_2_0_2, v, acc[60]);
    acc[61] = fma(m_1_3_0, v, acc[61]);
    acc[62] = fma(m_1_2_1, v, acc[62]);
    acc[63] = fma(m_1_1_2, v, acc[63]);
    acc[64] = fma(m_1_0_3, v, acc[64]);
    acc[65] = fma(py4, v, acc[65]);
    acc[66] = fma(m_0_3_1, v, acc[66]);
    acc[67] = fma(m_0_2_2, v, acc[67]);
    acc[68] = fma(m_0_1_3, v, acc[68]);
    acc[69] = fma(pz4, v, acc[69]);
  }
  { const T v = Mc[4];
    acc[4] = fma(T(1), v, acc[4]);
    acc[10] = fma(px1, v, acc[10]);
    acc[12] = fma(py1, v, acc[12]);
    acc[13] = fma(pz1, v, acc[13]);
    acc[20] = fma(px2, v, acc[20]);
    acc[22] = fma(m_1_1_0, v, acc[22]);
    acc[23] = fma(m_1_0_1, v, acc[23]);
    acc[25] = fma(py2, v, acc[25]);
    acc[26] = fma(m_0_1_1, v, acc[26]);
    acc[27] = fma(pz2, v, acc[27]);
    acc[35] = fma(px3, v, acc[35]);
    acc[37] = fma(m_2_1_0, v, acc[37]);
    acc[38] = fma(m_2_0_1, v, acc[38]);
    acc[40] = fma(m_1_2_0, v, acc[40]);
    acc[41] = fma(m_1_1_1, v, acc[41]);
    acc[42] = fma(m_1_0_2, v, acc[42]);
    acc[44] = fma(py3, v, acc[44]);
    acc[45] = fma(m_0_2_1, v, acc[45]);
    acc[46] = fma(m_0_1_2, v, acc[46]);
    acc[47] = fma(pz3, v, acc[47]);
    acc[56] = fma(px4, v, acc[56]);
    acc[58] = fma(m_3_1_0, v, acc[58]);
    acc[59] = fma(m_3_0_1, v, acc[59]);
    acc[61] = fma(m_2_2_0, v, acc[61]);
    acc[62] = fma(m_2_1_1, v, acc[62]);
    acc[63] = fma(m_2_0_2, v, acc[63]);
    acc[65] = fma(m_1_3_0, v, acc[65]);
    acc[66] = fma(m_1_2_1, v, acc[66]);
    acc[67] = fma(m_1_1_2, v, acc[67]);
    acc[68] = fma(m_1_0_3, v, acc[68]);
    acc[70] = fma(py4, v, acc[70]);
    acc[71] = fma(m_0_3_1, v, acc[71]);
    acc[72] = fma(m_0_2_2, v, acc[72]);
    acc[73] = fma(m_0_1_3, v, acc[73]);
    acc[74] = fma(pz4, v, acc[74]);
  }
  { const T v = Mc[5];
    acc[5] = fma(T(1), v, acc[5]);
    acc[11] = fma(px1, v, acc[11]);
    acc[13] = fma(py1, v, acc[13]);
    acc[14] = fma(pz1, v, acc[14]);
    acc[21] = fma(px2, v, acc[21]);
    acc[23] = fma(m_1_1_0, v, acc[23]);
    acc[24] = fma(m_1_0_1, v, acc[24]);
    acc[26] = fma(py2, v, acc[26]);
    acc[27] = fma(m_0_1_1, v, acc[27]);
    acc[28] = fma(pz2, v, acc[28]);
    acc[36] = fma(px3, v, acc[36]);
    acc[38] = fma(m_2_1_0, v, acc[38]);
    acc[39] = fma(m_2_0_1, v, acc[39]);
    acc[41] = fma(m_1_2_0, v, acc[41]);
    acc[42] = fma(m_1_1_1, v, acc[42]);
    acc[43] = fma(m_1_0_2, v, acc[43]);
    acc[45] = fma(py3, v, acc[45]);
    acc[46] = fma(m_0_2_1, v, acc[46]);
    acc[47] = fma(m_0_1_2, v, acc[47]);
    acc[48] = fma(pz3, v, acc[48]);
    acc[57] = fma(px4, v, acc[57]);
    acc[59] = fma(m_3_1_0, v, acc[59]);
    acc[60] = fma(m_3_0_1, v, acc[60]);
    acc[62] = fma(m_2_2_0, v, acc[62]);
    acc[63] = fma(m_2_1_1, v, acc[63]);
    acc[64] = fma(m_2_0_2, v, acc[64]);
    acc[66] = fma(m_1_3_0, v, acc[66]);
    acc[67] = fma(m_1_2_1, v, acc[67]);
    acc[68] = fma(m_1_1_2, v, acc[68]);
    acc[69] = fma(m_1_0_3, v, acc[69]);
    acc[71] = fma(py4, v, acc[71]);
    acc[72] = fma(m_0_3_1, v, acc[72]);
    acc[73] = fma(m_0_2_2, v, acc[73]);
    acc[74] = fma(m_0_1_3, v, acc[74]);
    acc[75] = fma(pz4, v, acc[75]);
  }
  { const T v = Mc[6];
    acc[6] = fma(T(1), v, acc[6]);
    acc[12] = fma(px1, v, acc[12]);
    acc[15] = fma(py1, v, acc[15]);
    acc[16] = fma(pz1, v, acc[16]);
    acc[22] = fma(px2, v, acc[22]);
    acc[25] = fma(m_1_1_0, v, acc[25]);
    acc[26] = fma(m_1_0_1, v, acc[26]);
    acc[29] = fma(py2, v, acc[29]);
    acc[30] = fma(m_0_1_1, v, acc[30]);
    acc[31] = fma(pz2, v, acc[31]);
    acc[37] = fma(px3, v, acc[37]);
    acc[40] = fma(m_2_1_0, v, acc[40]);
    acc[41] = fma(m_2_0_1, v, acc[41]);
    acc[44] = fma(m_1_2_0, v, acc[44]);
    acc[45] = fma(m_1_1_1, v, acc[45]);
    acc[46] = fma(m_1_0_2, v, acc[46]);
    acc[49] = fma(py3, v, acc[49]);
    acc[50] = fma(m_0_2_1, v, acc[50]);
    acc[51] = fma(m_0_1_2, v, acc[51]);
    acc[52] = fma(pz3, v, acc[52]);
    acc[58] = fma(px4, v, acc[58]);
    acc[61] = fma(m_3_1_0, v, acc[61]);
    acc[62] = fma(m_3_0_1, v, acc[62]);
    acc[65] = fma(m_2_2_0, v, acc[65]);
    acc[66] = fma(m_2_1_1, v, acc[66]);
    acc[67] = fma(m_2_0_2, v, acc[67]);
    acc[70] = fma(m_1_3_0, v, acc[70]);
    acc[71] = fma(m_1_2_1, v, acc[71]);
    acc[72] = fma(m_1_1_2, v, acc[72]);
    acc[73] = fma(m_1_0_3, v, acc[73]);
    acc[76] = fma(py4, v, acc[76]);
    acc[77] = fma(m_0_3_1, v, acc[77]);
    acc[78] = fma(m_0_2_2, v, acc[78]);
    acc[79] = fma(m_0_1_3, v, acc[79]);
    acc[80] = fma(pz4, v, acc[80]);
  }
  { const T v = Mc[7];
    acc[7] = fma(T(1), v, acc[7]);
    acc[13] = fma(px1, v, acc[13]);
    acc[16] = fma(py1, v, acc[16]);
    acc[17] = fma(pz1, v, acc[17]);
    acc[23] = fma(px2, v, acc[23]);
    acc[26] = fma(m_1_1_0, v, acc[26]);
    acc[27] = fma(m_1_0_1, v, acc[27]);
    acc[30] = fma(py2, v, acc[30]);
    acc[31] = fma(m_0_1_1, v, acc[31]);
    acc[32] = fma(pz2, v, acc[32]);
    acc[38] = fma(px3, v, acc[38]);
    acc[41] = fma(m_2_1_0, v, acc[41]);
    acc[42] = fma(m_2_0_1, v, acc[42]);
    acc[45] = fma(m_1_2_0, v, acc[45]);
    acc[46] = fma(m_1_1_1, v, acc[46]);
    acc[47] = fma(m_1_0_2, v, acc[47]);
    acc[50] = fma(py3, v, acc[50]);
    acc[51] = fma(m_0_2_1, v, acc[51]);
    acc[52] = fma(m_0_1_2, v, acc[52]);
    acc[53] = fma(pz3, v, acc[53]);
    acc[59] = fma(px4, v, acc[59]);
    acc[62] = fma(m_3_1_0, v, acc[62]);
    acc[63] = fma(m_3_0_1, v, acc[63]);
    acc[66] = fma(m_2_2_0, v, acc[66]);
    acc[67] = fma(m_2_1_1, v, acc[67]);
    acc[68] = fma(m_2_0_2, v, acc[68]);
    acc[71] = fma(m_1_3_0, v, acc[71]);
    acc[72] = fma(m_1_2_1, v, acc[72]);
    acc[73] = fma(m_1_1_2, v, acc[73]);
    acc[74] = fma(m_1_0_3, v, acc[74]);
    acc[77] = fma(py4, v, acc[77]);
    acc[78] = fma(m_0_3_1, v, acc[78]);
    acc[79] = fma(m_0_2_2, v, acc[79]);
    acc[80] = fma(m_0_1_3, v, acc[80]);
    acc[81] = fma(pz4, v, acc[81]);
  }
  { const T v = Mc[8];
    acc[8] = fma(T(1), v, acc[8]);
    acc[14] = fma(px1, v, acc[14]);
    acc[17] = fma(py1, v, acc[17]);
    acc[18] = fma(pz1, v, acc[18]);
    acc[24] = fma(px2, v, acc[24]);
    acc[27] = fma(m_1_1_0, v, acc[27]);
    acc[28] = fma(m_1_0_1, v, acc[28]);
    acc[31] = fma(py2, v, acc[31]);
    acc[32] = fma(m_0_1_1, v, acc[32]);
    acc[33] = fma(pz2, v, acc[33]);
    acc[39] = fma(px3, v, acc[39]);
    acc[42] = fma(m_2_1_0, v, acc[42]);
    acc[43] = fma(m_2_0_1, v, acc[43]);
    acc[46] = fma(m_1_2_0, v, acc[46]);
    acc[47] = fma(m_1_1_1, v, acc[47]);
    acc[48] = fma(m_1_0_2, v, acc[48]);
    acc[51] = fma(py3, v, acc[51]);
    acc[52] = fma(m_0_2_1, v, acc[52]);
    acc[53] = fma(m_0_1_2, v, acc[53]);
    acc[54] = fma(pz3, v, acc[54]);
    acc[60] = fma(px4, v, acc[60]);
    acc[63] = fma(m_3_1_0, v, acc[63]);
    acc[64] = fma(m_3_0_1, v, acc[64]);
    acc[67] = fma(m_2_2_0, v, acc[67]);
    acc[68] = fma(m_2_1_1, v, acc[68]);
    acc[69] = fma(m_2_0_2, v, acc[69]);
    acc[72] = fma(m_1_3_0, v, acc[72]);
    acc[73] = fma(m_1_2_1, v, acc[73]);
    acc[74] = fma(m_1_1_2, v, acc[74]);
    acc[75] = fma(m_1_0_3, v, acc[75]);
    acc[78] = fma(py4, v, acc[78]);
    acc[79] = fma(m_0_3_1, v, acc[79]);
    acc[80] = fma(m_0_2_2, v, acc[80]);
    acc[81] = fma(m_0_1_3, v, acc[81]);
    acc[82] = fma(pz4, v, acc[82]);
  }
  { const T v = Mc[9];
    acc[9] = fma(T(1), v, acc[9]);
    acc[19] = fma(px1, v, acc[19]);
    acc[20] = fma(py1, v, acc[20]);
    acc[21] = fma(pz1, v, acc[21]);
    acc[34] = fma(px2, v, acc[34]);
    acc[35] = fma(m_1_1_0, v, acc[35]);
    acc[36] = fma(m_1_0_1, v, acc[36]);
    acc[37] = fma(py2, v, acc[37]);
    acc[38] = fma(m_0_1_1, v, acc[38]);
    acc[39] = fma(pz2, v, acc[39]);
    acc[55] = fma(px3, v, acc[55]);
    acc[56] = fma(m_2_1_0, v, acc[56]);
    acc[57] = fma(m_2_0_1, v, acc[57]);
    acc[58] = fma(m_1_2_0, v, acc[58]);
    acc[59] = fma(m_1_1_1, v, acc[59]);
    acc[60] = fma(m_1_0_2, v, acc[60]);
    acc[61] = fma(py3, v, acc[61]);
    acc[62] = fma(m_0_2_1, v, acc[62]);
    acc[63] = fma(m_0_1_2, v, acc[63]);
    acc[64] = fma(pz3, v, acc[64]);
  }
  { const T v = Mc[10];
    acc[10] = fma(T(1), v, acc[10]);
    acc[20] = fma(px1, v, acc[20]);
    acc[22] = fma(py1, v, acc[22]);
    acc[23] = fma(pz1, v, acc[23]);
    acc[35] = fma(px2, v, acc[35]);
    acc[37] = fma(m_1_1_0, v, acc[37]);
    acc[38] = fma(m_1_0_1, v, acc[38]);
    acc[40] = fma(py2, v, acc[40]);
    acc[41] = fma(m_0_1_1, v, acc[41]);
    acc[42] = fma(pz2, v, acc[42]);
    acc[56] = fma(px3, v, acc[56]);
    acc[58] = fma(m_2_1_0, v, acc[58]);
    acc[59] = fma(m_2_0_1, v, acc[59]);
    acc[61] = fma(m_1_2_0, v, acc[61]);
    acc[62] = fma(m_1_1_1, v, acc[62]);
    acc[63] = fma(m_1_0_2, v, acc[63]);
    acc[65] = fma(py3, v, acc[65]);
    acc[66] = fma(m_0_2_1, v, acc[66]);
    acc[67] = fma(m_0_1_2, v, acc[67]);
    acc[68] = fma(pz3, v, acc[68]);
  }
  { const T v = Mc[11];
    acc[11] = fma(T(1), v, acc[11]);
    acc[21] = fma(px1, v, acc[21]);
    acc[23] = fma(py1, v, acc[23]);
    acc[24] = fma(pz1, v, acc[24]);
    acc[36] = fma(px2, v, acc[36]);
    acc[38] = fma(m_1_1_0, v, acc[38]);
    acc[39] = fma(m_1_0_1, v, acc[39]);
    acc[41] = fma(py2, v, acc[41]);
    acc[42] = fma(m_0_1_1, v, acc[42]);
    acc[43] = fma(pz2, v, acc[43]);
    acc[57] = fma(px3, v, acc[57]);
    acc[59] = fma(m_2_1_0, v, acc[59]);
    acc[60] = fma(m_2_0_1, v, acc[60]);
    acc[62] = fma(m_1_2_0, v, acc[62]);
    acc[63] = fma(m_1_1_1, v, acc[63]);
    acc[64] = fma(m_1_0_2, v, acc[64]);
    acc[66] = fma(py3, v, acc[66]);
    acc[67] = fma(m_0_2_1, v, acc[67]);
    acc[68] = fma(m_0_1_2, v, acc[68]);
    acc[69] = fma(pz3, v, acc[69]);
  }
  { const T v = Mc[12];
    acc[12] = fma(T(1), v, acc[12]);
    acc[22] = fma(px1, v, acc[22]);
    acc[25] = fma(py1, v, acc[25]);
    acc[26] = fma(pz1, v, acc[26]);
    acc[37] = fma(px2, v, acc[37]);
    acc[40] = fma(m_1_1_0, v, acc[40]);
    acc[41] = fma(m_1_0_1, v, acc[41]);
    acc[44] = fma(py2, v, acc[44]);
    acc[45] = fma(m_0_1_1, v, acc[45]);
    acc[46] = fma(pz2, v, acc[46]);
    acc[58] = fma(px3, v, acc[58]);
    acc[61] = fma(m_2_1_0, v, acc[61]);
    acc[62] = fma(m_2_0_1, v, acc[62]);
    acc[65] = fma(m_1_2_0, v, acc[65]);
    acc[66] = fma(m_1_1_1, v, acc[66]);
    acc[67] = fma(m_1_0_2, v, acc[67]);
    acc[70] = fma(py3, v, acc[70]);
    acc[71] = fma(m_0_2_1, v, acc[71]);
    acc[72] = fma(m_0_1_2, v, acc[72]);
    acc[73] = fma(pz3, v, acc[73]);
  }
  { const T v = Mc[13];
    acc[13] = fma(T(1), v, acc[13]);
    acc[23] = fma(px1, v, acc[23]);
    acc[26] = fma(py1, v, acc[26]);
    acc[27] = fma(pz1, v, acc[27]);
    acc[38] = fma(px2, v, acc[38]);
    acc[41] = fma(m_1_1_0, v, acc[41]);
    acc[42] = fma(m_1_0_1, v, acc[42]);
    acc[45] = fma(py2, v, acc[45]);
    acc[46] = fma(m_0_1_1, v, acc[46]);
    acc[47] = fma(pz2, v, acc[47]);
    acc[59] = fma(px3, v, acc[59]);
    acc[62] = fma(m_2_1_0, v, acc[62]);
    acc[63] = fma(m_2_0_1, v, acc[63]);
    acc[66] = fma(m_1_2_0, v, acc[66]);
    acc[67] = fma(m_1_1_1, v, acc[67]);
    acc[68] = fma(m_1_0_2, v, acc[68]);
    acc[71] = fma(py3, v, acc[71]);
    acc[72] = fma(m_0_2_1, v, acc[72]);
    acc[73] = fma(m_0_1_2, v, acc[73]);
    acc[74] = fma(pz3, v, acc[74]);
  }
  { const T v = Mc[14];
    acc[14] = fma(T(1), v, acc[14]);
    acc[24] = fma(px1, v, acc[24]);
    acc[27] = fma(py1, v, acc[27]);
    acc[28] = fma(pz1, v, acc[28]);
    acc[39] = fma(px2, v, acc[39]);
    acc[42] = fma(m_1_1_0, v, acc[42]);
    acc[43] = fma(m_1_0_1, v, acc[43]);
    acc[46] = fma(py2, v, acc[46]);
    acc[47] = fma(m_0_1_1, v, acc[47]);
    acc[48] = fma(pz2, v, acc[48]);
    acc[60] = fma(px3, v, acc[60]);
    acc[63] = fma(m_2_1_0, v, acc[63]);
    acc[64] = fma(m_2_0_1, v, acc[64]);
    acc[67] = fma(m_1_2_0, v, acc[67]);
    acc[68] = fma(m_1_1_1, v, acc[68]);
    acc[69] = fma(m_1_0_2, v, acc[69]);
    acc[72] = fma(py3, v, acc[72]);
    acc[73] = fma(m_0_2_1, v, acc[73]);
    acc[74] = fma(m_0_1_2, v, acc[74]);
    acc[75] = fma(pz3, v, acc[75]);
  }
  { const T v = Mc[15];
    acc[15] = fma(T(1), v, acc[15]);
    acc[25] = fma(px1, v, acc[25]);
    acc[29] = fma(py1, v, acc[29]);
    acc[30] = fma(pz1, v, acc[30]);
    acc[40] = fma(px2, v, acc[40]);
    acc[44] = fma(m_1_1_0, v, acc[44]);
    acc[45] = fma(m_1_0_1, v, acc[45]);
    acc[49] = fma(py2, v, acc[49]);
    acc[50] = fma(m_0_1_1, v, acc[50]);
    acc[51] = fma(pz2, v, acc[51]);
    acc[61] = fma(px3, v, acc[61]);
    acc[65] = fma(m_2_1_0, v, acc[65]);
    acc[66] = fma(m_2_0_1, v, acc[66]);
    acc[70] = fma(m_1_2_0, v, acc[70]);
    acc[71] = fma(m_1_1_1, v, acc[71]);
    acc[72] = fma(m_1_0_2, v, acc[72]);
    acc[76] = fma(py3, v, acc[76]);
    acc[77] = fma(m_0_2_1, v, acc[77]);
    acc[78] = fma(m_0_1_2, v, acc[78]);
    acc[79] = fma(pz3, v, acc[79]);
  }
  { const T v = Mc[16];
    acc[16] = fma(T(1), v, acc[16]);
    acc[26] = fma(px1, v, acc[26]);
    acc[30] = fma(py1, v, acc[30]);
    acc[31] = fma(pz1, v, acc[31]);
    acc[41] = fma(px2, v, acc[41]);
    acc[45] = fma(m_1_1_0, v, acc[45]);
    acc[46] = fma(m_1_0_1, v, acc[46]);
    acc[50] = fma(py2, v, acc[50]);
    acc[51] = fma(m_0_1_1, v, acc[51]);
    acc[52] = fma(pz2, v, acc[52]);
    acc[62] = fma(px3, v, acc[62]);
    acc[66] = fma(m_2_1_0, v, acc[66]);
    acc[67] = fma(m_2_0_1, v, acc[67]);
    acc[71] = fma(m_1_2_0, v, acc[71]);
    acc[72] = fma(m_1_1_1, v, acc[72]);
    acc[73] = fma(m_1_0_2, v, acc[73]);
    acc[77] = fma(py3, v, acc[77]);
    acc[78] = fma(m_0_2_1, v, acc[78]);
    acc[79] = fma(m_0_1_2, v, acc[79]);
    acc[80] = fma(pz3, v, acc[80]);
  }
  { const T v = Mc[17];
    acc[17] = fma(T(1), v, acc[17]);
    acc[27] = fma(px1, v, acc[27]);
    acc[31] = fma(py1, v, acc[31]);
    acc[32] = fma(pz1, v, acc[32]);
    acc[42] = fma(px2, v, acc[42]);
    acc[46] = fma(m_1_1_0, v, acc[46]);
    acc[47] = fma(m_1_0_1, v, acc[47]);
    acc[51] = fma(py2, v, acc[51]);
    acc[52] = fma(m_0_1_1, v, acc[52]);
    acc[53] = fma(pz2, v, acc[53]);
    acc[63] = fma(px3, v, acc[63]);
    acc[67] = fma(m_2_1_0, v, acc[67]);
    acc[68] = fma(m_2_0_1, v, acc[68]);
    acc[72] = fma(m_1_2_0, v, acc[72]);
    acc[73] = fma(m_1_1_1, v, acc[73]);
    acc[74] = fma(m_1_0_2, v, acc[74]);
    acc[78] = fma(py3, v, acc[78]);
    acc[79] = fma(m_0_2_1, v, acc[79]);
    acc[80] = fma(m_0_1_2, v, acc[80]);
    acc[81] = fma(pz3, v, acc[81]);
  }
  { const T v = Mc[18];
    acc[18] = fma(T(1), v, acc[18]);
    acc[28] = fma(px1, v, acc[28]);
    acc[32] = fma(py1, v, acc[32]);
    acc[33] = fma(pz1, v, acc[33]);
    acc[43] = fma(px2, v, acc[43]);
    acc[47] = fma(m_1_1_0, v, acc[47]);
    acc[48] = fma(m_1_0_1, v, acc[48]);
    acc[52] = fma(py2, v, acc[52]);
    acc[53] = fma(m_0_1_1, v, acc[53]);
    acc[54] = fma(pz2, v, acc[54]);
    acc[64] = fma(px3, v, acc[64]);
    acc[68] = fma(m_2_1_0, v, acc[68]);
    acc[69] = fma(m_2_0_1, v, acc[69]);
    acc[73] = fma(m_1_2_0, v, acc[73]);
    acc[74] = fma(m_1_1_1, v, acc[74]);
    acc[75] = fma(m_1_0_2, v, acc[75]);
    acc[79] = fma(py3, v, acc[79]);
    acc[80] = fma(m_0_2_1, v, acc[80]);
    acc[81] = fma(m_0_1_2, v, acc[81]);
    acc[82] = fma(pz3, v, acc[82]);
  }
  { const T v = Mc[19];
    acc[19] = fma(T(1), v, acc[19]);
    acc[34] = fma(px1, v, acc[34]);
    acc[35] = fma(py1, v, acc[35]);
    acc[36] = fma(pz1, v, acc[36]);
    acc[55] = fma(px2, v, acc[55]);
    acc[56] = fma(m_1_1_0, v, acc[56]);
    acc[57] = fma(m_1_0_1, v, acc[57]);
    acc[58] = fma(py2, v, acc[58]);
    acc[59] = fma(m_0_1_1, v, acc[59]);
    acc[60] = fma(pz2, v, acc[60]);
  }
  { const T v = Mc[20];
    acc[20] = fma(T(1), v, acc[20]);
    acc[35] = fma(px1, v, acc[35]);
    acc[37] = fma(py1, v, acc[37]);
    acc[38] = fma(pz1, v, acc[38]);
    acc[56] = fma(px2, v, acc[56]);
    acc[58] = fma(m_1_1_0, v, acc[58]);
    acc[59] = fma(m_1_0_1, v, acc[59]);
    acc[61] = fma(py2, v, acc[61]);
    acc[62] = fma(m_0_1_1, v, acc[62]);
    acc[63] = fma(pz2, v, acc[63]);
  }
  { const T v = Mc[21];
    acc[21] = fma(T(1), v, acc[21]);
    acc[36] = fma(px1, v, acc[36]);
    acc[38] = fma(py1, v, acc[38]);
    acc[39] = fma(pz1, v, acc[39]);
    acc[57] = fma(px2, v, acc[57]);
    acc[59] = fma(m_1_1_0, v, acc[59]);
    acc[60] = fma(m_1_0_1, v, acc[60]);
    acc[62] = fma(py2, v, acc[62]);
    acc[63] = fma(m_0_1_1, v, acc[63]);
    acc[64] = fma(pz2, v, acc[64]);
  }
  { const T v = Mc[22];
    acc[22] = fma(T(1), v, acc[22]);
    acc[37] = fma(px1, v, acc[37]);
    acc[40] = fma(py1, v, acc[40]);
    acc[41] = fma(pz1, v, acc[41]);
    acc[58] = fma(px2, v, acc[58]);
    acc[61] = fma(m_1_1_0, v, acc[61]);
    acc[62] = fma(m_1_0_1, v, acc[62]);
    acc[65] = fma(py2, v, acc[65]);
    acc[66] = fma(m_0_1_1, v, acc[66]);
    acc[67] = fma(pz2, v, acc[67]);
  }
  { const T v = Mc[23];
    acc[23] = fma(T(1), v, acc[23]);
    acc[38] = fma(px1, v, acc[38]);
    acc[41] = fma(py1, v, acc[41]);
    acc[42] = fma(pz1, v, acc[42]);
    acc[59] = fma(px2, v, acc[59]);
    acc[62] = fma(m_1_1_0, v, acc[62]);
    acc[63] = fma(m_1_0_1, v, acc[63]);
    acc[66] = fma(py2, v, acc[66]);
    acc[67] = fma(m_0_1_1, v, acc[67]);
    acc[68] = fma(pz2, v, acc[68]);
  }
  { const T v = Mc[24];
    acc[24] = fma(T(1), v, acc[24]);
    acc[39] = fma(px1, v, acc[39]);
    acc[42] = fma(py1, v, acc[42]);
    acc[43] = fma(pz1, v, acc[43]);
    acc[60] = fma(px2, v, acc[60]);
    acc[63] = fma(m_1_1_0, v, acc[63]);
    acc[64] = fma(m_1_0_1, v, acc[64]);
    acc[67] = fma(py2, v, acc[67]);
    acc[68] = fma(m_0_1_1, v, acc[68]);
    acc[69] = fma(pz2, v, acc[69]);
  }
  { const T v = Mc[25];
    acc[25] = fma(T(1), v, acc[25]);
    acc[40] = fma(px1, v, acc[40]);
    acc[44] = fma(py1, v, acc[44]);
    acc[45] = fma(pz1, v, acc[45]);
    acc[61] = fma(px2, v, acc[61]);
    acc[65] = fma(m_1_1_0, v, acc[65]);
    acc[66] = fma(m_1_0_1, v, acc[66]);
    acc[70] = fma(py2, v, acc[70]);
    acc[71] = fma(m_0_1_1, v, acc[71]);
    acc[72] = fma(pz2, v, acc[72]);
  }
  { const T v = Mc[26];
    acc[26] = fma(T(1), v, acc[26]);
    acc[41] = fma(px1, v, acc[41]);
    acc[45] = fma(py1, v, acc[45]);
    acc[46] = fma(pz1, v, acc[46]);
    acc[62] = fma(px2, v, acc[62]);
    acc[66] = fma(m_1_1_0, v, acc[66]);
    acc[67] = fma(m_1_0_1, v, acc[67]);
    acc[71] = fma(py2, v, acc[71]);
    acc[72] = fma(m_0_1_1, v, acc[72]);
    acc[73] = fma(pz2, v, acc[73]);
  }
  { const T v = Mc[27];
    acc[27] = fma(T(1), v, acc[27]);
    acc[42] = fma(px1, v, acc[42]);
    acc[46] = fma(py1, v, acc[46]);
    acc[47] = fma(pz1, v, acc[47]);
    acc[63] = fma(px2, v, acc[63]);
    acc[67] = fma(m_1_1_0, v, acc[67]);
    acc[68] = fma(m_1_0_1, v, acc[68]);
    acc[72] = fma(py2, v, acc[72]);
    acc[73] = fma(m_0_1_1, v, acc[73]);
    acc[74] = fma(pz2, v, acc[74]);
  }
  { const T v = Mc[28];
    acc[28] = fma(T(1), v, acc[28]);
    acc[43] = fma(px1, v, acc[43]);
    acc[47] = fma(py1, v, acc[47]);
    acc[48] = fma(pz1, v, acc[48]);
    acc[64] = fma(px2, v, acc[64]);
    acc[68] = fma(m_1_1_0, v, acc[68]);
    acc[69] = fma(m_1_0_1, v, acc[69]);
    acc[73] = fma(py2, v, acc[73]);
    acc[74] = fma(m_0_1_1, v, acc[74]);
    acc[75] = fma(pz2, v, acc[75]);
  }
  { const T v = Mc[29];
    acc[29] = fma(T(1), v, acc[29]);
    acc[44] = fma(px1, v, acc[44]);
    acc[49] = fma(py1, v, acc[49]);
    acc[50] = fma(pz1, v, acc[50]);
    acc[65] = fma(px2, v, acc[65]);
    acc[70] = fma(m_1_1_0, v, acc[70]);
    acc[71] = fma(m_1_0_1, v, acc[71]);
    acc[76] = fma(py2, v, acc[76]);
    acc[77] = fma(m_0_1_1, v, acc[77]);
    acc[78] = fma(pz2, v, acc[78]);
  }
  { const T v = Mc[30];
    acc[30] = fma(T(1), v, acc[30]);
    acc[45] = fma(px1, v, acc[45]);
    acc[50] = fma(py1, v, acc[50]);
    acc[51] = fma(pz1, v, acc[51]);
    acc[66] = fma(px2, v, acc[66]);
    acc[71] = fma(m_1_1_0, v, acc[71]);
    acc[72] = fma(m_1_0_1, v, acc[72]);
    acc[77] = fma(py2, v, acc[77]);
    acc[78] = fma(m_0_1_1, v, acc[78]);
    acc[79] = fma(pz2, v, acc[79]);
  }
  { const T v = Mc[31];
    acc[31] = fma(T(1), v, acc[31]);
    acc[46] = fma(px1, v, acc[46]);
    acc[51] = fma(py1, v, acc[51]);
    acc[52] = fma(pz1, v, acc[52]);
    acc[67] = fma(px2, v, acc[67]);
    acc[72] = fma(m_1_1_0, v, acc[72]);
    acc[73] = fma(m_1_0_1, v, acc[73]);
    acc[78] = fma(py2, v, acc[78]);
    acc[79] = fma(m_0_1_1, v, acc[79]);
    acc[80] = fma(pz2, v, acc[80]);
  }
  { const T v = Mc[32];
    acc[32] = fma(T(1), v, acc[32]);
    acc[47] = fma(px1, v, acc[47]);
    acc[52] = fma(py1, v, acc[52]);
    acc[53] = fma(pz1, v, acc[53]);
    acc[68] = fma(px2, v, acc[68]);
    acc[73] = fma(m_1_1_0, v, acc[73]);
    acc[74] = fma(m_1_0_1, v, acc[74]);
    acc[79] = fma(py2, v, acc[79]);
    acc[80] = fma(m_0_1_1, v, acc[80]);
    acc[81] = fma(pz2, v, acc[81]);
  }
  { const T v = Mc[33];
    acc[33] = fma(T(1), v, acc[33]);
    acc[48] = fma(px1, v, acc[48]);
    acc[53] = fma(py1, v, acc[53]);
    acc[54] = fma(pz1, v, acc[54]);
    acc[69] = fma(px2, v, acc[69]);
    acc[74] = fma(m_1_1_0, v, acc[74]);
    acc[75] = fma(m_1_0_1, v, acc[75]);
    acc[80] = fma(py2, v, acc[80]);
    acc[81] = fma(m_0_1_1, v, acc[81]);
    acc[82] = fma(pz2, v, acc[82]);
  }
  { const T v = Mc[34];
    acc[34] = fma(T(1), v, acc[34]);
    acc[55] = fma(px1, v, acc[55]);
    acc[56] = fma(py1, v, acc[56]);
    acc[57] = fma(pz1, v, acc[57]);
  }
  { const T v = Mc[35];
    acc[35] = fma(T(1), v, acc[35]);
    acc[56] = fma(px1, v, acc[56]);
    acc[58] = fma(py1, v, acc[58]);
    acc[59] = fma(pz1, v, acc[59]);
  }
  { const T v = Mc[36];
    acc[36] = fma(T(1), v, acc[36]);
    acc[57] = fma(px1, v, acc[57]);
    acc[59] = fma(py1, v, acc[59]);
    acc[60] = fma(pz1, v, acc[60]);
  }
  { const T v = Mc[37];
    acc[37] = fma(T(1), v, acc[37]);
    acc[58] = fma(px1, v, acc[58]);
    acc[61] = fma(py1, v, acc[61]);
    acc[62] = fma(pz1, v, acc[62]);
  }
  { const T v = Mc[38];
    acc[38] = fma(T(1), v, acc[38]);
    acc[59] = fma(px1, v, acc[59]);
    acc[62] = fma(py1, v, acc[62]);
    acc[63] = fma(pz1, v, acc[63]);
  }
  { const T v = Mc[39];
    acc[39] = fma(T(1), v, acc[39]);
    acc[60] = fma(px1, v, acc[60]);
    acc[63] = fma(py1, v, acc[63]);
    acc[64] = fma(pz1, v, acc[64]);
  }
  { const T v = Mc[40];
    acc[40] = fma(T(1), v, acc[40]);
    acc[61] = fma(px1, v, acc[61]);
    acc[65] = fma(py1, v, acc[65]);
    acc[66] = fma(pz1, v, acc[66]);
  }
  { const T v = Mc[41];
    acc[41] = fma(T(1), v, acc[41]);
    acc[62] = fma(px1, v, acc[62]);
    acc[66] = fma(py1, v, acc[66]);
    acc[67] = fma(pz1, v, acc[67]);
  }
  { const T v = Mc[42];
    acc[42] = fma(T(1), v, acc[42]);
    acc[63] = fma(px1, v, acc[63]);
    acc[67] = fma(py1, v, acc[67]);
    acc[68] = fma(pz1, v, acc[68]);
  }
  { const T v = Mc[43];
    acc[43] = fma(T(1), v, acc[43]);
    acc[64] = fma(px1, v, acc[64]);
    acc[68] = fma(py1, v, acc[68]);
    acc[69] = fma(pz1, v, acc[69]);
  }
  { const T v = Mc[44];
    acc[44] = fma(T(1), v, acc[44]);
    acc[65] = fma(px1, v, acc[65]);
    acc[70] = fma(py1, v, acc[70]);
    acc[71] = fma(pz1, v, acc[71]);
  }
  { const T v = Mc[45];
    acc[45] = fma(T(1), v, acc[45]);
    acc[66] = fma(px1, v, acc[66]);
    acc[71] = fma(py1, v, acc[71]);
    acc[72] = fma(pz1, v, acc[72]);
  }
  { const T v = Mc[46];
    acc[46] = fma(T(1), v, acc[46]);
    acc[67] = fma(px1, v, acc[67]);
    acc[72] = fma(py1, v, acc[72]);
    acc[73] = fma(pz1, v, acc[73]);
  }
  { const T v = Mc[47];
    acc[47] = fma(T(1), v, acc[47]);
    acc[68] = fma(px1, v, acc[68]);
    acc[73] = fma(py1, v, acc[73]);
    acc[74] = fma(pz1, v, acc[74]);
  }
  { const T v = Mc[48];
    acc[48] = fma(T(1), v, acc[48]);
    acc[69] = fma(px1, v, acc[69]);
    acc[74] = fma(py1, v, acc[74]);
    acc[75] = fma(pz1, v, acc[75]);
  }
  { const T v = Mc[49];
    acc[49] = fma(T(1), v, acc[49]);
    acc[70] = fma(px1, v, acc[70]);
    acc[76] = fma(py1, v, acc[76]);
    acc[77] = fma(pz1, v, acc[77]);
  }
  { const T v = Mc[50];
    acc[50] = fma(T(1), v, acc[50]);
    acc[71] = fma(px1, v, acc[71]);
    acc[77] = fma(py1, v, acc[77]);
    acc[78] = fma(pz1, v, acc[78]);
  }
  { const T v = Mc[51];
    acc[51] = fma(T(1), v, acc[51]);
    acc[72] = fma(px1, v, acc[72]);
    acc[78] = fma(py1, v, acc[78]);
    acc[79] = fma(pz1, v, acc[79]);
  }
  { const T v = Mc[52];
    acc[52] = fma(T(1), v, acc[52]);
    acc[73] = fma(px1, v, acc[73]);
    acc[79] = fma(py1, v, acc[79]);
    acc[80] = fma(pz1, v, acc[80]);
  }
  { const T v = Mc[53];
    acc[53] = fma(T(1), v, acc[53]);
    acc[74] = fma(px1, v, acc[74]);
    acc[80] = fma(py1, v, acc[80]);
    acc[81] = fma(pz1, v, acc[81]);
  }
  { const T v = Mc[54];
    acc[54] = fma(T(1), v, acc[54]);
    acc[75] = fma(px1, v, acc[75]);
    acc[81] = fma(py1, v, acc[81]);
    acc[82] = fma(pz1, v, acc[82]);
  }
  { const T v = Mc[55];
    acc[55] = fma(T(1), v, acc[55]);
  }
  { const T v = Mc[56];
    acc[56] = fma(T(1), v, acc[56]);
  }
  { const T v = Mc[57];
    acc[57] = fma(T(1), v, acc[57]);
  }
  { const T v = Mc[58];
    acc[58] = fma(T(1), v, acc[58]);
  }
  { const T v = Mc[59];
    acc[59] = fma(T(1), v, acc[59]);
  }
  { const T v = Mc[60];
    acc[60] = fma(T(1), v, acc[60]);
  }
  { const T v = Mc[61];
    acc[61] = fma(T(1), v, acc[61]);
  }
  { const T v = Mc[62];
    acc[62] = fma(T(1), v, acc[62]);
  }
  { const T v = Mc[63];
    acc[63] = fma(T(1), v, acc[63]);
  }
  { const T v = Mc[64];
    acc[64] = fma(T(1), v, acc[64]);
  }
  { const T v = Mc[65];
    acc[65] = fma(T(1), v, acc[65]);
  }
  { const T v = Mc[66];
    acc[66] = fma(T(1), v, acc[66]);
  }
  { const T v = Mc[67];
    acc[67] = fma(T(1), v, acc[67]);
  }
  { const T v = Mc[68];
    acc[68] = fma(T(1), v, acc[68]);
  }
  { const T v = Mc[69];
    acc[69] = fma(T(1), v, acc[69]);
  }
  { const T v = Mc[70];
    acc[70] = fma(T(1), v, acc[70]);
  }
  { const T v = Mc[71];
    acc[71] = fma(T(1), v, acc[71]);
  }
  { const T v = Mc[72];
    acc[72] = fma(T(1), v, acc[72]);
  }
  { const T v = Mc[73];
    acc[73] = fma(T(1), v, acc[73]);
  }
  { const T v = Mc[74];
    acc[74] = fma(T(1), v, acc[74]);
  }
  { const T v = Mc[75];
    acc[75] = fma(T(1), v, acc[75]);
  }
  { const T v = Mc[76];
    acc[76] = fma(T(1), v, acc[76]);
  }
  { const T v = Mc[77];
    acc[77] = fma(T(1), v, acc[77]);
  }
  { const T v = Mc[78];
    acc[78] = fma(T(1), v, acc[78]);
  }
  { const T v = Mc[79];
    acc[79] = fma(T(1), v, acc[79]);
  }
  { const T v = Mc[80];
    acc[80] = fma(T(1), v, acc[80]);
  }
  { const T v = Mc[81];
    acc[81] = fma(T(1), v, acc[81]);
  }
  { const T v = Mc[82];
    acc[82] = fma(T(1), v, acc[82]);
  }
}
// L2L: local expansion Lc about a centre at -(x, y, z) from this one, order 6
template <typename T>
__device__ __forceinline__ void l2l_m1_p6(T x, T y, T z, const T* __restrict__ Lc, T* __restrict__ acc) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T px5 = px4 * x * cinv<T>(5);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T py5 = py4 * y * cinv<T>(5);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T pz5 = pz4 * z * cinv<T>(5);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  const T m_4_1_0 = px4 * py1;
  const T m_4_0_1 = px4 * pz1;
  const T m_3_2_0 = px3 * py2;
  const T m_3_1_1 = px3 * py1 * pz1;
  const T m_3_0_2 = px3 * pz2;
  const T m_2_3_0 = px2 * py3;
  const T m_2_2_1 = px2 * py2 * pz1;
  const T m_2_1_2 = px2 * py1 * pz2;
  const T m_2_0_3 = px2 * pz3;
  const T m_1_4_0 = px1 * py4;
  const T m_1_3_1 = px1 * py3 * pz1;
  const T m_1_2_2 = px1 * py2 * pz2;
  const T m_1_1_3 = px1 * py1 * pz3;
  const T m_1_0_4 = px1 * pz4;
  const T m_0_4_1 = py4 * pz1;
  const T m_0_3_2 = py3 * pz2;
  const T m_0_2_3 = py2 * pz3;
  const T m_0_1_4 = py1 * pz4;
  { const T v = Lc[0];
    acc[0] = fma(T(1), v, acc[0]);
  }
  { const T v = Lc[1];
    acc[0] = fma(px1, v, acc[0]);
    acc[1] = fma(T(1), v, acc[1]);
  }
  { const T v = Lc[2];
    acc[0] = fma(py1, v, acc[0]);
    acc[2] = fma(T(1), v, acc[2]);
  }
  { const T v = Lc[3];
    acc[0] = fma(pz1, v, acc[0]);
    acc[3] = fma(T(1), v, acc[3]);
  }
  { const T v = Lc[4];
    acc[0] = fma(px2, v, acc[0]);
    acc[1] = fma(px1, v, acc[1]);
    acc[4] = fma(T(1), v, acc[4]);
  }
  { const T v = Lc[5];
    acc[0] = fma(m_1_1_0, v, acc[0]);
    acc[1] = fma(py1, v, acc[1]);
    acc[2] = fma(px1, v, acc[2]);
    acc[5] = fma(T(1), v, acc[5]);
  }
  { const T v = Lc[6];
    acc[0] = fma(m_1_0_1, v, acc[0]);
    acc[1] = fma(pz1, v, acc[1]);
    acc[3] = fma(px1, v, acc[3]);
    acc[6] = fma(T(1), v, acc[6]);
  }
  { const T v = Lc[7];
    acc[0] = fma(py2, v, acc[0]);
    acc[2] = fma(py1, v, acc[2]);
    acc[7] = fma(T(1), v, acc[7]);
  }
  { const T v = Lc[8];
    acc[0] = fma(m_0_1_1, v, acc[0]);
    acc[2] = fma(pz1, v, acc[2]);
    acc[3] = fma(py1, v, acc[3]);
    acc[8] = fma(T(1), v, acc[8]);
  }
  { const T v = Lc[9];
    acc[0] = fma(pz2, v, acc[0]);
    acc[3] = fma(pz1, v, acc[3]);
    acc[9] = fma(T(1), v, acc[9]);
  }
  { const T v = Lc[10];
    acc[0] = fma(px3, v, acc[0]);
    acc[1] = fma(px2, v, acc[1]);
    acc[4] = fma(px1, v, acc[4]);
    acc[10] = fma(T(1), v, acc[10]);
  }
  { const T v = Lc[11];
    acc[0] = fma(m_2_1_0, v, acc[0]);
    acc[1] = fma(m_1_1_0, v, acc[1]);
    acc[2] = fma(px2, v, acc[2]);
    acc[4] = fma(py1, v, acc[4]);
    acc[5] = fma(px1, v, acc[5]);
    acc[11] = fma(T(1), v, acc[11]);
  }
  { const T v = Lc[12];
    acc[0] = fma(m_2_0_1, v, acc[0]);
    acc[1] = fma(m_1_0_1, v, acc[1]);
    acc[3] = fma(px2, v, acc[3]);
    acc[4] = fma(pz1, v, acc[4]);
    acc[6] = fma(px1, v, acc[6]);
    acc[12] = fma(T(1), v, acc[12]);
  }
  { const T v = Lc[13];
    acc[0] = fma(m_1_2_0, v, acc[0]);
    acc[1] = fma(py2, v, acc[1]);
    acc[2] = fma(m_1_1_0, v, acc[2]);
    acc[5] = fma(py1, v, acc[5]);
    acc[7] = fma(px1, v, acc[7]);
    acc[13] = fma(T(1), v, acc[13]);
  }
  { const T v = Lc[14];
    acc[0] = fma(m_1_1_1, v, acc[0]);
    acc[1] = fma(m_0_1_1, v, acc[1]);
    acc[2] = fma(m_1_0_1, v, acc[2]);
    acc[3] = fma(m_1_1_0, v, acc[3]);
    acc[5] = fma(pz1, v, acc[5]);
    acc[6] = fma(py1, v, acc[6]);
    acc[8] = fma(px1, v, acc[8]);
    acc[14] = fma(T(1), v, acc[14]);
  }
  { const T v = Lc[15];
    acc[0] = fma(m_1_0_2, v, acc[0]);
    acc[1] = fma(pz2, v, acc[1]);
    acc[3] = fma(m_1_0_1, v, acc[3]);
    acc[6] = fma(pz1, v, acc[6]);
    acc[9] = fma(px1, v, acc[9]);
    acc[15] = fma(T(1), v, acc[15]);
  }
  { const T v = Lc[16];
    acc[0] = fma(py3, v, acc[0]);
    acc[2] = fma(py2, v, acc[2]);
    acc[7] = fma(py1, v, acc[7]);
    acc[16] = fma(T(1), v, acc[16]);
  }
  { const T v = Lc[17];
    acc[0] = fma(m_0_2_1, v, acc[0]);
    acc[2] = fma(m_0_1_1, v, acc[2]);
    acc[3] = fma(py2, v, acc[3]);
    acc[7] = fma(pz1, v, acc[7]);
    acc[8] = fma(py1, v, acc[8]);
    acc[17] = fma(T(1), v, acc[17]);
  }
  { const T v = Lc[18];
    acc[0] = fma(m_0_1_2, v, acc[0]);
    acc[2] = fma(pz2, v, acc[2]);
    acc[3] = fma(m_0_1_1, v, acc[3]);
    acc[8] = fma(pz1, v, acc[8]);
    acc[9] = fma(py1, v, acc[9]);
    acc[18] = fma(T(1), v, acc[18]);
  }
  { const T v = Lc[19];
    acc[0] = fma(pz3, v, acc[0]);
    acc[3] = fma(pz2, v, acc[3]);
    acc[9] = fma(pz1, v, acc[9]);
    acc[19] = fma(T(1), v, acc[19]);
  }
  { const T v = Lc[20];
    acc[0] = fma(px4, v, acc[0]);
    acc[1] = fma(px3, v, acc[1]);
    acc[4] = fma(px2, v, acc[4]);
    acc[10] = fma(px1, v, acc[10]);
    acc[20] = fma(T(1), v, acc[20]);
  }
  { const T v = Lc[21];
    acc[0] = fma(m_3_1_0, v, acc[0]);
    acc[1] = fma(m_2_1_0, v, acc[1]);
    acc[2] = fma(px3, v, acc[2]);
    acc[4] = fma(m_1_1_0, v, acc[4]);
    acc[5] = fma(px2, v, acc[5]);
    acc[10] = fma(py1, v, acc[10]);
    acc[11] = fma(px1, v, acc[11]);
    acc[21] = fma(T(1), v, acc[21]);
  }
  { const T v = Lc[22];
    acc[0] = fma(m_3_0_1, v, acc[0]);
    acc[1] = fma(m_2_0_1, v, acc[1]);
    acc[3] = fma(px3, v, acc[3]);
    acc[4] = fma(m_1_0_1, v, acc[4]);
    acc[6] = fma(px2, v, acc[6]);
    acc[10] = fma(pz1, v, acc[10]);
    acc[12] = fma(px1, v, acc[12]);
    acc[22] = fma(T(1), v, acc[22]);
  }
  { const T v = Lc[23];
    acc[0] = fma(m_2_2_0, v, acc[0]);
    acc[1] = fma(m_1_2_0, v, acc[1]);
    acc[2] = fma(m_2_1_0, v, acc[2]);
    acc[4] = fma(py2, v, acc[4]);
    acc[5] = fma(m_1_1_0, v, acc[5]);
    acc[7] = fma(px2, v, acc[7]);
    acc[11] = fma(py1, v, acc[11]);
    acc[13] = fma(px1, v, acc[13]);
    acc[23] = fma(T(1), v, acc[23]);
  }
  { const T v = Lc[24];
    acc[0] = fma(m_2_1_1, v, acc[0]);
    acc[1] = fma(m_1_1_1, v, acc[1]);
    acc[2] = fma(m_2_0_1, v, acc[2]);
    acc[3] = fma(m_2_1_0, v, acc[3]);
    acc[4] = fma(m_0_1_1, v, acc[4]);
    acc[5] = fma(m_1_0_1, v, acc[5]);
    acc[6] = fma(m_1_1_0, v, acc[6]);
    acc[8] = fma(px2, v, acc[8]);
    acc[11] = fma(pz1, v, acc[11]);
    acc[12] = fma(py1, v, acc[12]);
    acc[14] = fma(px1, v, acc[14]);
    acc[24] = fma(T(1), v, acc[24]);
  }
  { const T v = Lc[25];
    acc[0] = fma(m_2_0_2, v, acc[0]);
    acc[1] = fma(m_1_0_2, v, acc[1]);
    acc[3] = fma(m_2_0_1, v, acc[3]);
    acc[4] = fma(pz2, v, acc[4]);
    acc[6] = fma(m_1_0_1, v, acc[6]);
    acc[9] = fma(px2, v, acc[9]);
    acc[12] = fma(pz1, v, acc[12]);
    acc[15] = fma(px1, v, acc[15]);
    acc[25] = fma(T(1), v, acc[25]);
  }
  { const T v = Lc[26];
    acc[0] = fma(m_1_3_0, v, acc[0]);
    acc[1] = fma(py3, v, acc[1]);
    acc[2] = fma(m_1_2_0, v, acc[2]);
    acc[5] = fma(py2, v, acc[5]);
    acc[7] = fma(m_1_1_0, v, acc[7]);
    acc[13] = fma(py1, v, acc[13]);
    acc[16] = fma(px1, v, acc[16]);
    acc[26] = fma(T(1), v, acc[26]);
  }
  { const T v = Lc[27];
    acc[0] = fma(m_1_2_1, v, acc[0]);
    acc[1] = fma(m_0_2_1, v, acc[1]);
    acc[2] = fma(m_1_1_1, v, acc[2]);
    acc[3] = fma(m_1_2_0, v, acc[3]);
    acc[5] = fma(m_0_1_1, v, acc[5]);
    acc[6] = fma(py2, v, acc[6]);
    acc[7] = fma(m_1_0_1, v, acc[7]);
    acc[8] = fma(m_1_1_0, v, acc[8]);
    acc[13] = fma(pz1, v, acc[13]);
    acc[14] = fma(py1, v, acc[14]);
    acc[17] = fma(px1, v, acc[17]);
    acc[27] = fma(T(1), v, acc[27]);
  }
  { const T v = Lc[28];
    acc[0] = fma(m_1_1_2, v, acc[0]);
    acc[1] = fma(m_0_1_2, v, acc[1]);
    acc[2] = fma(m_1_0_2, v, acc[2]);
    acc[3] = fma(m_1_1_1, v, acc[3]);
    acc[5] = fma(pz2, v, acc[5]);
    acc[6] = fma(m_0_1_1, v, acc[6]);
    acc[8] = fma(m_1_0_1, v, acc[8]);
    acc[9] = fma(m_1_1_0, v, acc[9]);
    acc[14] = fma(pz1, v, acc[14]);
    acc[15] = fma(py1, v, acc[15]);
    acc[18] = fma(px1, v, acc[18]);
    acc[28] = fma(T(1), v, acc[28]);
  }
  { const T v = Lc[29];
    acc[0] = fma(m_1_0_3, v, acc[0]);
    acc[1] = fma(pz3, v, acc[1]);
    acc[3] = fma(m_1_0_2, v, acc[3]);
    acc[6] = fma(pz2, v, acc[6]);
    acc[9] = fma(m_1_0_1, v, acc[9]);
    acc[15] = fma(pz1, v, acc[15]);
    acc[19] = fma(px1, v, acc[19]);
    acc[29] = fma(T(1), v, acc[29]);
  }
  { const T v = Lc[30];
    acc[0] = fma(py4, v, acc[0]);
    acc[2] = fma(py3, v, acc[2]);
    acc[7] = fma(py2, v, acc[7]);
    acc[16] = fma(py1, v, acc[16]);
    acc[30] = fma(T(1), v, acc[30]);
  }
  { const T v = Lc[31];
    acc[0] = fma(m_0_3_1, v, acc[0]);
    acc[2] = fma(m_0_2_1, v, acc[2]);
    acc[3] = fma(py3, v, acc[3]);
    acc[7] = fma(m_0_1_1, v, acc[7]);
    acc[8] = fma(py2, v, acc[8]);
    acc[16] = fma(pz1, v, acc[16]);
    acc[17] = fma(py1, v, acc[17]);
    acc[31] = fma(T(1), v, acc[31]);
  }
  { const T v = Lc[32];
    acc[0] = fma(m_0_2_2, v, acc[0]);
    acc[2] = fma(m_0_1_2, v, acc[2]);
    acc[3] = fma(m_0_2_1, v, acc[3]);
    acc[7] = fma(pz2, v, acc[7]);
    acc[8] = fma(m_0_1_1, v, acc[8]);
    acc[9] = fma(py2, v, acc[9]);
    acc[17] = fma(pz1, v, acc[17]);
    acc[18] = fma(py1, v, acc[18]);
    acc[32] = fma(T(1), v, acc[32]);
  }
  { const T v = Lc[33];
    acc[0] = fma(m_0_1_3, v, acc[0]);
    acc[2] = fma(pz3, v, acc[2]);
    acc[3] = fma(m_0_1_2, v, acc[3]);
    acc[8] = fma(pz2, v, acc[8]);
    acc[9] = fma(m_0_1_1, v, acc[9]);
    acc[18] = fma(pz1, v, acc[18]);
    acc[19] = fma(py1, v, acc[19]);
    acc[33] = fma(T(1), v, acc[33]);
  }
  { const T v = Lc[34];
    acc[0] = fma(pz4, v, acc[0]);
    acc[3] = fma(pz3, v, acc[3]);
    acc[9] = fma(pz2, v, acc[9]);
    acc[19] = fma(pz1, v, acc[19]);
    acc[34] = fma(T(1), v, acc[34]);
  }
  { const T v = Lc[35];
    acc[0] = fma(px5, v, acc[0]);
    acc[1] = fma(px4, v, acc[1]);
    acc[4] = fma(px3, v, acc[4]);
    acc[10] = fma(px2, v, acc[10]);
    acc[20] = fma(px1, v, acc[20]);
    acc[35] = fma(T(1), v, acc[35]);
  }
  { const T v = Lc[36];
    acc[0] = fma(m_4_1_0, v, acc[0]);
    acc[1] = fma(m_3_1_0, v, acc[1]);
    acc[2] = fma(px4, v, acc[2]);
    acc[4] = fma(m_2_1_0, v, acc[4]);
    acc[5] = fma(px3, v, acc[5]);
    acc[10] = fma(m_1_1_0, v, acc[10]);
    acc[11] = fma(px2, v, acc[11]);
    acc[20] = fma(py1, v, acc[20]);
    acc[21] = fma(px1, v, acc[21]);
    acc[36] = fma(T(1), v, acc[36]);
  }
  { const T v = Lc[37];
    acc[0] = fma(m_4_0_1, v, acc[0]);
    acc[1] = fma(m_3_0_1, v, acc[1]);
    acc[3] = fma(px4, v, acc[3]);
    acc[4] = fma(m_2_0_1, v, acc[4]);
    acc[6] = fma(px3, v, acc[6]);
    acc[10] = fma(m_1_0_1, v, acc[10]);
    acc[12] = fma(px2, v, acc[12]);
    acc[20] = fma(pz1, v, acc[20]);
    acc[22] = fma(px1, v, acc[22]);
    acc[37] = fma(T(1), v, acc[37]);
  }
  { const T v = Lc[38];
    acc[0] = fma(m_3_2_0, v, acc[0]);
    acc[1] = fma(m_2_2_0, v, acc[1]);
    acc[2] = fma(m_3_1_0, v, acc[2]);
    acc[4] = fma(m_1_2_0, v, acc[4]);
    acc[5] = fma(m_2_1_0, v, acc[5]);
    acc[7] = fma(px3, v, acc[7]);
    acc[10] = fma(py2, v, acc[10]);
    acc[11] = fma(m_1_1_0, v, acc[11]);
    acc[13] = fma(px2, v, acc[13]);
    acc[21] = fma(py1, v, acc[21]);
    acc[23] = fma(px1, v, acc[23]);
    acc[38] = fma(T(1), v, acc[38]);
  }
  { const T v = Lc[39];
    acc[0] = fma(m_3_1_1, v, acc[0]);
    acc[1] = fma(m_2_1_1, v, acc[1]);
    acc[2] = fma(m_3_0_1, v, acc[2]);
    acc[3] = fma(m_3_1_0, v, acc[3]);
    acc[4] = fma(m_1_1_1, v, acc[4]);
    acc[5] = fma(m_2_0_1, v, acc[5]);
    acc[6] = fma(m_2_1_0, v, acc[6]);
    acc[8] = fma(px3, v, acc[8]);
    acc[10] = fma(m_0_1_1, v, acc[10]);
    acc[11] = fma(m_1_0_1, v, acc[11]);
    acc[12] = fma(m_1_1_0, v, acc[12]);
    acc[14] = fma(px2, v, acc[14]);
    acc[21] = fma(pz1, v, acc[21]);
    acc[22] = fma(py1, v, acc[22]);
    acc[24] = fma(px1, v, acc[24]);
    acc[39] = fma(T(1), v, acc[39]);
  }
  { const T v = Lc[40];
    acc[0] = fma(m_3_0_2, v, acc[0]);
    acc[1] = fma(m_2_0_2, v, acc[1]);
    acc[3] = fma(m_3_0_1, v, acc[3]);
    acc[4] = fma(m_1_0_2, v, acc[4]);
    acc[6] = fma(m_2_0_1, v, acc[6]);
    acc[9] = fma(px3, v, acc[9]);
    acc[10] = fma(pz2, v, acc[10]);
    acc[12] = fma(m_1_0_1, v, acc[12]);
    acc[15] = fma(px2, v, acc[15]);
    acc[22] = fma(pz1, v, acc[22]);
    acc[25] = fma(px1, v, acc[25]);
    acc[40] = fma(T(1), v, acc[40]);
  }
  { const T v = Lc[41];
    acc[0] = fma(m_2_3_0, v, acc[0]);
    acc[1] = fma(m_1_3_0, v, acc[1]);
    acc[2] = fma(m_2_2_0, v, acc[2]);
    acc[4] = fma(py3, v, acc[4]);
    acc[5] = fma(m_1_2_0, v, acc[5]);
    acc[7] = fma(m_2_1_0, v, acc[7]);
    acc[11] = fma(py2, v, acc[11]);
    acc[13] = fma(m_1_1_0, v, acc[13]);
    acc[16] = fma(px2, v, acc[16]);
    acc[23] = fma(py1, v, acc[23]);
    acc[26] = fma(px1, v, acc[26]);
    acc[41] = fma(T(1), v, acc[41]);
  }
  { const T v = Lc[42];
    acc[0] = fma(m_2_2_1, v, acc[0]);
    acc[1] = fma(m_1_2_1, v, acc[1]);
    acc[2] = fma(m_2_1_1, v, acc[2]);
    acc[3] = fma(m_2_2_0, v, acc[3]);
    acc[4] = fma(m_0_2_1, v, acc[4]);
    acc[5] = fma(m_1_1_1, v, acc[5]);
    acc[6] = fma(m_1_2_0, v, acc[6]);
    acc[7] = fma(m_2_0_1, v, acc[7]);
    acc[8] = fma(m_2_1_0, v, acc[8]);
    acc[11] = fma(m_0_1_1, v, acc[11]);
    acc[12] = fma(py2, v, acc[12]);
    acc[13] = fma(m_1_0_1, v, acc[13]);
    acc[14] = fma(m_1_1_0, v, acc[14]);
    acc[17] = fma(px2, v, acc[17]);
    acc[23] = fma(pz1, v, acc[23]);
    acc[24] = fma(py1, v, acc[24]);
    acc[27] = fma(px1, v, acc[27]);
    acc[42] = fma(T(1), v, acc[42]);
  }
  { const T v = Lc[43];
    acc[0] = fma(m_2_1_2, v, acc[0]);
    acc[1] = fma(m_1_1_2, v, acc[1]);
    acc[2] = fma(m_2_0_2, v, acc[2]);
    acc[3] = fma(m_2_1_1, v, acc[3]);
    acc[4] = fma(m_0_1_2, v, acc[4]);
    acc[5] = fma(m_1_0_2, v, acc[5]);
    acc[6] = fma(m_1_1_1, v, acc[6]);
    acc[8] = fma(m_2_0_1, v, acc[8]);
    acc[9] = fma(m_2_1_0, v, acc[9]);
    acc[11] = fma(pz2, v, acc[11]);
    acc[12] = fma(m_0_1_1, v, acc[12]);
    acc[14] = fma(m_1_0_1, v, acc[14]);
    acc[15] = fma(m_1_1_0, v, acc[15]);
    acc[18] = fma(px2, v, acc[18]);
    acc[24] = fma(pz1, v, acc[24]);
    acc[25] = fma(py1, v, acc[25]);
    acc[28] = fma(px1, v, acc[28]);
    acc[43] = fma(T(1), v, acc[43]);
  }
  { const T v = Lc[44];
    acc[0] = fma(m_2_0_3, v, acc[0]);
    acc[1] = fma(m_1_0_3, v, acc[1]);
    acc[3] = fma(m_2_0_2, v, acc[3]);
    acc[4] = fma(pz3, v, acc[4]);
    acc[6] = fma(m_1_0_2, v, acc[6]);
    acc[9] = fma(m_2_0_1, v, acc[9]);
    acc[12] = fma(pz2, v, acc[12]);
    acc[15] = fma(m_1_0_1, v, acc[15]);
    acc[19] = fma(px2, v, acc[19]);
    acc[25] = fma(pz1, v, acc[25]);
    acc[29] = fma(px1, v, acc[29]);
    acc[44] = fma(T(1), v, acc[44]);
  }
  { const T v = Lc[45];
    acc[0] = fma(m_1_4_0, v, acc[0]);
    acc[1] = fma(py4, v, acc[1]);
    acc[2] = fma(m_1_3_0, v, acc[2]);
    acc[5] = fma(py3, v, acc[5]);
    acc[7] = fma(m_1_2_0, v, acc[7]);
    acc[13] = fma(py2, v, acc[13]);
    acc[16] = fma(m_1_1_0, v, acc[16]);
    acc[26] = fma(py1, v, acc[26]);
    acc[30] = fma(px1, v, acc[30]);
    acc[45] = fma(T(1), v, acc[45]);
  }
  { const T v = Lc[46];
    acc[0] = fma(m_1_3_1, v, acc[0]);
    acc[1] = fma(m_0_3_1, v, acc[1]);
    acc[2] = fma(m_1_2_1, v, acc[2]);
    acc[3] = fma(m_1_3_0, v, acc[3]);
    acc[5] = fma(m_0_2_1, v, acc[5]);
    acc[6] = fma(py3, v, acc[6]);
    acc[7] = fma(m_1_1_1, v, acc[7]);
    acc[8] = fma(m_1_2_0, v, acc[8]);
    acc[13] = fma(m_0_1_1, v, acc[13]);
    acc[14] = fma(py2, v, acc[14]);
    acc[16] = fma(m_1_0_1, v, acc[16]);
    acc[17] = fma(m_1_1_0, v, acc[17]);
    acc[26] = fma(pz1, v, acc[26]);
    acc[27] = fma(py1, v, acc[27]);
    acc[31] = fma(px1, v, acc[31]);
    acc[46] = fma(T(1), v, acc[46]);
  }
  { const T v = Lc[47];
    acc[0] = fma(m_1_2_2, v, acc[0]);
    acc[1] = fma(m_0_2_2, v, acc[1]);
    acc[2] = fma(m_1_1_2, v, acc[2]);
    acc[3] = fma(m_1_2_1, v, acc[3]);
    acc[5] = fma(m_0_1_2, v, acc[5]);
    acc[6] = fma(m_0_2_1, v, acc[6]);
    acc[7] = fma(m_1_0_2, v, acc[7]);
    acc[8] = fma(m_1_1_1, v, acc[8]);
    acc[9] = fma(m_1_2_0, v, acc[9]);
    acc[13] = fma(pz2, v, acc[13]);
    acc[14] = fma(m_0_1_1, v, acc[14]);
    acc[15] = fma(py2, v, acc[15]);
    acc[17] = fma(m_1_0_1, v, acc[17]);
    acc[18] = fma(m_1_1_0, v, acc[18]);
    acc[27] = fma(pz1, v, acc[27]);
    acc[28] = fma(py1, v, acc[28]);
    acc[32] = fma(px1, v, acc[32]);
    acc[47] = fma(T(1), v, acc[47]);
  }
  { const T v = Lc[48];
    acc[0] = fma(m_1_1_3, v, acc[0]);
    acc[1] = fma(m_0_1_3, v, acc[1]);
    acc[2] = fma(m_1_0_3, v, acc[2]);
    acc[3] = fma(m_1_1_2, v, acc[3]);
    acc[5] = fma(pz3, v, acc[5]);
    acc[6] = fma(m_0_1_2, v, acc[6]);
    acc[8] = fma(m_1_0_2, v, acc[8]);
    acc[9] = fma(m_1_1_1, v, acc[9]);
    acc[14] = fma(pz2, v, acc[14]);
    acc[15] = fma(m_0_1_1, v, acc[15]);
    acc[18] = fma(m_1_0_1, v, acc[18]);
    acc[19] = fma(m_1_1_0, v, acc[19]);
    acc[28] = fma(pz1, v, acc[28]);
    acc[29] = fma(py1, v, acc[29]);
    acc[33] = fma(px1, v, acc[33]);
    acc[48] = fma(T(1), v, acc[48]);
  }
  { const T v = Lc[49];
    acc[0] = fma(m_1_0_4, v, acc[0]);
    acc[1] = fma(pz4, v, acc[1]);
    acc[3] = fma(m_1_0_3, v, acc[3]);
    acc[6] = fma(pz3, v, acc[6]);
    acc[9] = fma(m_1_0_2, v, acc[9]);
    acc[15] = fma(pz2, v, acc[15]);
    acc[19] = fma(m_1_0_1, v, acc[19]);
    acc[29] = fma(pz1, v, acc[29]);
    acc[34] = fma(px1, v, acc[34]);
    acc[49] = fma(T(1), v, acc[49]);
  }
  { const T v = Lc[50];
    acc[0] = fma(py5, v, acc[0]);
    acc[2] = fma(py4, v, acc[2]);
    acc[7] = fma(py3, v, acc[7]);
    acc[16] = fma(py2, v, acc[16]);
    acc[30] = fma(py1, v, acc[30]);
    acc[50] = fma(T(1), v, acc[50]);
  }
  { const T v = Lc[51];
    acc[0] = fma(m_0_4_1, v, acc[0]);
    acc[2] = fma(m_0_3_1, v, acc[2]);
    acc[3] = fma(py4, v, acc[3]);
    acc[7] = fma(m_0_2_1, v, acc[7]);
    acc[8] = fma(py3, v, acc[8]);
    acc[16] = fma(m_0_1_1, v, acc[16]);
    acc[17] = fma(py2, v, acc[17]);
    acc[30] = fma(pz1, v, acc[30]);
    acc[31] = fma(py1, v, acc[31]);
    acc[51] = fma(T(1), v, acc[51]);
  }
  { const T v = Lc[52];
    acc[0] = fma(m_0_3_2, v, acc[0]);
    acc[2] = fma(m_0_2_2, v, acc[2]);
    acc[3] = fma(m_0_3_1, v, acc[3]);
    acc[7] = fma(m_0_1_2, v, acc[7]);
    acc[8] = fma(m_0_2_1, v, acc[8]);
    acc[9] = fma(py3, v, acc[9]);
    acc[16] = fma(pz2, v, acc[16]);
    acc[17] = fma(m_0_1_1, v, acc[17]);
    acc[18] = fma(py2, v, acc[18]);
    acc[31] = fma(pz1, v, acc[31]);
    acc[32] = fma(py1, v, acc[32]);
    acc[52] = fma(T(1), v, acc[52]);
  }
  { const T v = Lc[53];
    acc[0] = fma(m_0_2_3, v, acc[0]);
    acc[2] = fma(m_0_1_3, v, acc[2]);
    acc[3] = fma(m_0_2_2, v, acc[3]);
    acc[7] = fma(pz3, v, acc[7]);
    acc[8] = fma(m_0_1_2, v, acc[8]);
    acc[9] = fma(m_0_2_1, v, acc[9]);
    acc[17] = fma(pz2, v, acc[17]);
    acc[18] = fma(m_0_1_1, v, acc[18]);
    acc[19] = fma(py2, v, acc[19]);
    acc[32] = fma(pz1, v, acc[32]);
    acc[33] = fma(py1, v, acc[33]);
    acc[53] = fma(T(1), v, acc[53]);
  }
  { const T v = Lc[54];
    acc[0] = fma(m_0_1_4, v, acc[0]);
    acc[2] = fma(pz4, v, acc[2]);
    acc[3] = fma(m_0_1_3, v, acc[3]);
    acc[8] = fma(pz3, v, acc[8]);
    acc[9] = fma(m_0_1_2, v, acc[9]);
    acc[18] = fma(pz2, v, acc[18]);
    acc[19] = fma(m_0_1_1, v, acc[19]);
    acc[33] = fma(pz1, v, acc[33]);
    acc[34] = fma(py1, v, acc[34]);
    acc[54] = fma(T(1), v, acc[54]);
  }
  { const T v = Lc[55];
    acc[0] = fma(pz5, v, acc[0]);
    acc[3] = fma(pz4, v, acc[3]);
    acc[9] = fma(pz3, v, acc[9]);
    acc[19] = fma(pz2, v, acc[19]);
    acc[34] = fma(pz1, v, acc[34]);
    acc[55] = fma(T(1), v, acc[55]);
  }
}
// L2P: field -grad of the local expansion Lc at offset (x, y, z) = site - centre, order 6
template <typename T>
__device__ __forceinline__ void l2p_m1_p6(T x, T y, T z, const T* __restrict__ Lc, T& f0, T& f1, T& f2) {
  const T px1 = x;
  const T px2 = px1 * x * cinv<T>(2);
  const T px3 = px2 * x * cinv<T>(3);
  const T px4 = px3 * x * cinv<T>(4);
  const T py1 = y;
  const T py2 = py1 * y * cinv<T>(2);
  const T py3 = py2 * y * cinv<T>(3);
  const T py4 = py3 * y * cinv<T>(4);
  const T pz1 = z;
  const T pz2 = pz1 * z * cinv<T>(2);
  const T pz3 = pz2 * z * cinv<T>(3);
  const T pz4 = pz3 * z * cinv<T>(4);
  const T m_1_1_0 = px1 * py1;
  const T m_1_0_1 = px1 * pz1;
  const T m_0_1_1 = py1 * pz1;
  const T m_2_1_0 = px2 * py1;
  const T m_2_0_1 = px2 * pz1;
  const T m_1_2_0 = px1 * py2;
  const T m_1_1_1 = px1 * py1 * pz1;
  const T m_1_0_2 = px1 * pz2;
  const T m_0_2_1 = py2 * pz1;
  const T m_0_1_2 = py1 * pz2;
  const T m_3_1_0 = px3 * py1;
  const T m_3_0_1 = px3 * pz1;
  const T m_2_2_0 = px2 * py2;
  const T m_2_1_1 = px2 * py1 * pz1;
  const T m_2_0_2 = px2 * pz2;
  const T m_1_3_0 = px1 * py3;
  const T m_1_2_1 = px1 * py2 * pz1;
  const T m_1_1_2 = px1 * py1 * pz2;
  const T m_1_0_3 = px1 * pz3;
  const T m_0_3_1 = py3 * pz1;
  const T m_0_2_2 = py2 * pz2;
  const T m_0_1_3 = py1 * pz3;
  { const T v = -Lc[1];
    f0 = fma(T(1), v, f0);
  }
  { const T v = -Lc[2];
    f1 = fma(T(1), v, f1);
  }
  { const T v = -Lc[3];
    f2 = fma(T(1), v, f2);
  }
  { const T v = -Lc[4];
    f0 = fma(px1, v, f0);
  }
  { const T v = -Lc[5];
    f0 = fma(py1, v, f0);
    f1 = fma(px1, v, f1);
  }
  { const T v = -Lc[6];
    f0 = fma(pz1, v, f0);
    f2 = fma(px1, v, f2);
  }
  { const T v = -Lc[7];
    f1 = fma(py1, v, f1);
  }
  { const T v = -Lc[8];
    f1 = fma(pz1, v, f1);
    f2 = fma(py1, v, f2);
  }
  { const T v = -Lc[9];
    f2 = fma(pz1, v, f2);
  }
  { const T v = -Lc[10];
    f0 = fma(px2, v, f0);
  }
  { const T v = -Lc[11];
    f0 = fma(m_1_1_0, v, f0);
    f1 = fma(px2, v, f1);
  }
  { const T v = -Lc[12];
    f0 = fma(m_1_0_1, v, f0);
    f2 = fma(px2, v, f2);
  }
  { const T v = -Lc[13];
    f0 = fma(py2, v, f0);
    f1 = fma(m_1_1_0, v, f1);
  }
  { const T v = -Lc[14];
    f0 = fma(m_0_1_1, v, f0);
    f1 = fma(m_1_0_1, v, f1);
    f2 = fma(m_1_1_0, v, f2);
  }
  { const T v = -Lc[15];
    f0 = fma(pz2, v, f0);
    f2 = fma(m_1_0_1, v, f2);
  }
  { const T v = -Lc[16];
    f1 = fma(py2, v, f1);
  }
  { const T v = -Lc[17];
    f1 = fma(m_0_1_1, v, f1);
    f2 = fma(py2, v, f2);
  }
  { const T v = -Lc[18];
    f1 = fma(pz2, v, f1);
    f2 = fma(m_0_1_1, v, f2);
  }
  { const T v = -Lc[19];
    f2 = fma(pz2, v, f2);
  }
  { const T v = -Lc[20];
    f0 = fma(px3, v, f0);
  }
  { const T v = -Lc[21];
    f0 = fma(m_2_1_0, v, f0);
    f1 = fma(px3, v, f1);
  }
  { const T v = -Lc[22];
    f0 = fma(m_2_0_1, v, f0);
    f2 = fma(px3, v, f2);
  }
  { const T v = -Lc[23];
    f0 = fma(m_1_2_0, v, f0);
    f1 = fma(m_2_1_0, v, f1);
  }
  { const T v = -Lc[24];
    f0 = fma(m_1_1_1, v, f0);
    f1 = fma(m_2_0_1, v, f1);
    f2 = fma(m_2_1_0, v, f2);
  }
  { const T v = -Lc[25];
    f0 = fma(m_1_0_2, v, f0);
    f2 = fma(m_2_0_1, v, f2);
  }
  { const T v = -Lc[26];
    f0 = fma(py3, v, f0);
    f1 = fma(m_1_2_0, v, f1);
  }
  { const T v = -Lc[27];
    f0 = fma(m_0_2_1, v, f0);
    f1 = fma(m_1_1_1, v, f1);
    f2 = fma(m_1_2_0, v, f2);
  }
  { const T v = -Lc[28];
    f0 = fma(m_0_1_2, v, f0);
    f1 = fma(m_1_0_2, v, f1);
    f2 = fma(m_1_1_1, v, f2);
  }
  { const T v = -Lc[29];
    f0 = fma(pz3, v, f0);
    f2 = fma(m_1_0_2, v, f2);
  }
  { const T v = -Lc[30];
    f1 = fma(py3, v, f1);
  }
  { const T v = -Lc[31];
    f1 = fma(m_0_2_1, v, f1);
    f2 = fma(py3, v, f2);
  }
  { const T v = -Lc[32];
    f1 = fma(m_0_1_2, v, f1);
    f2 = fma(m_0_2_1, v, f2);
  }
  { const T v = -Lc[33];
    f1 = fma(pz3, v, f1);
    f2 = fma(m_0_1_2, v, f2);
  }
  { const T v = -Lc[34];
    f2 = fma(pz3, v, f2);
  }
  { const T v = -Lc[35];
    f0 = fma(px4, v, f0);
  }
  { const T v = -Lc[36];
    f0 = fma(m_3_1_0, v, f0);
    f1 = fma(px4, v, f1);
  }
  { const T v = -Lc[37];
    f0 = fma(m_3_0_1, v, f0);
    f2 = fma(px4, v, f2);
  }
  { const T v = -Lc[38];
    f0 = fma(m_2_2_0, v, f0);
    f1 = fma(m_3_1_0, v, f1);
  }
  { const T v = -Lc[39];
    f0 = fma(m_2_1_1, v, f0);
    f1 = fma(m_3_0_1, v, f1);
    f2 = fma(m_3_1_0, v, f2);
  }
  { const T v = -Lc[40];
    f0 = fma(m_2_0_2, v, f0);
    f2 = fma(m_3_0_1, v, f2);
  }
  { const T v = -Lc[41];
    f0 = fma(m_1_3_0, v, f0);
    f1 = fma(m_2_2_0, v, f1);
  }
  { const T v = -Lc[42];
    f0 = fma(m_1_2_1, v, f0);
    f1 = fma(m_2_1_1, v, f1);
    f2 = fma(m_2_2_0, v, f2);
  }
  { const T v = -Lc[43];
    f0 = fma(m_1_1_2, v, f0);
    f1 = fma(m_2_0_2, v, f1);
    f2 = fma(m_2_1_1, v, f2);
  }
  { const T v = -Lc[44];
    f0 = fma(m_1_0_3, v, f0);
    f2 = fma(m_2_0_2, v, f2);
  }
  { const T v = -Lc[45];
    f0 = fma(py4, v, f0);
    f1 = fma(m_1_3_0, v, f1);
  }
  { const T v = -Lc[46];
    f0 = fma(m_0_3_1, v, f0);
    f1 = fma(m_1_2_1, v, f1);
    f2 = fma(m_1_3_0, v, f2);
  }
  { const T v = -Lc[47];
    f0 = fma(m_0_2_2, v, f0);
    f1 = fma(m_1_1_2, v, f1);
    f2 = fma(m_1_2_1, v, f2);
  }
  { const T v = -Lc[48];
    f0 = fma(m_0_1_3, v, f0);
    f1 = fma(m_1_0_3, v, f1);
    f2 = fma(m_1_1_2, v, f2);
  }
  { const T v = -Lc[49];
    f0 = fma(pz4, v, f0);
    f2 = fma(m_1_0_3, v, f2);
  }
  { const T v = -Lc[50];
    f1 = fma(py4, v, f1);
  }
  { const T v = -Lc[51];
    f1 = fma(m_0_3_1, v, f1);
    f2 = fma(py4, v, f2);
  }
  { const T v = -Lc[52];
    f1 = fma(m_0_2_2, v, f1);
    f2 = fma(m_0_3_1, v, f2);
  }
  { const T v = -Lc[53];
    f1 = fma(m_0_1_3, v, f1);
    f2 = fma(m_0_2_2, v, f2);
  }
  { const T v = -Lc[54];
    f1 = fma(pz4, v, f1);
    f2 = fma(m_0_1_3, v, f2);
  }
  { const T v = -Lc[55];
    f2 = fma(pz4, v, f2);
  }
}

// loop-form tables of M2L, source order 1, expansion order 5
static __constant__ short m2l_rec_m1_p5[448] = {
  -1, -1, -1, -1, -1, -1, 0, 0, 0, -1, -1, -1, -1, -1, 1, 0, -1, 0, -1, -1, -1, -1, 1, 0, -1, -1, 0, -1, -1, -1, 1, 0, 1, -1, -1, 0, -1, -1, 2, 0, 2, 1, -1, -1, -1, -1, 2, 0, 3, -1, 1, -1, -1, -1, 2, 0, -1, 2, -1, -1, 0, -1, 2, 0, -1, 3, 2, -1, -1, -1, 2, 0, -1, -1, 3, -1, -1, 0, 2, 0, 4, -1, -1, 1, -1, -1, 3, 0, 5, 4, -1, 2, -1, -1, 3, 0, 6, -1, 4, 3, -1, -1, 3, 0, 7, 5, -1, -1, 1, -1, 3, 0, 8, 6, 5, -1, -1, -1, 3, 0, 9, -1, 6, -1, -1, 1, 3, 0, -1, 7, -1, -1, 2, -1, 3, 0, -1, 8, 7, -1, 3, -1, 3, 0, -1, 9, 8, -1, -1, 2, 3, 0, -1, -1, 9, -1, -1, 3, 3, 0, 10, -1, -1, 4, -1, -1, 4, 0, 11, 10, -1, 5, -1, -1, 4, 0, 12, -1, 10, 6, -1, -1, 4, 0, 13, 11, -1, 7, 4, -1, 4, 0, 14, 12, 11, 8, -1, -1, 4, 0, 15, -1, 12, 9, -1, 4, 4, 0, 16, 13, -1, -1, 5, -1, 4, 0, 17, 14, 13, -1, 6, -1, 4, 0, 18, 15, 14, -1, -1, 5, 4, 0, 19, -1, 15, -1, -1, 6, 4, 0, -1, 16, -1, -1, 7, -1, 4, 0, -1, 17, 16, -1, 8, -1, 4, 0, -1, 18, 17, -1, 9, 7, 4, 0, -1, 19, 18, -1, -1, 8, 4, 0, -1, -1, 19, -1, -1, 9, 4, 0, 20, -1, -1, 10, -1, -1, 5, 0, 21, 20, -1, 11, -1, -1, 5, 0, 22, -1, 20, 12, -1, -1, 5, 0, 23, 21, -1, 13, 10, -1, 5, 0, 24, 22, 21, 14, -1, -1, 5, 0, 25, -1, 22, 15, -1, 10, 5, 0, 26, 23, -1, 16, 11, -1, 5, 0, 27, 24, 23, 17, 12, -1, 5, 0, 28, 25, 24, 18, -1, 11, 5, 0, 29, -1, 25, 19, -1, 12, 5, 0, 30, 26, -1, -1, 13, -1, 5, 0, 31, 27, 26, -1, 14, -1, 5, 0, 32, 28, 27, -1, 15, 13, 5, 0, 33, 29, 28, -1, -1, 14, 5, 0, 34, -1, 29, -1, -1, 15, 5, 0, -1, 30, -1, -1, 16, -1, 5, 0, -1, 31, 30, -1, 17, -1, 5, 0, -1, 32, 31, -1, 18, 16, 5, 0, -1, 33, 32, -1, 19, 17, 5, 0, -1, 34, 33, -1, -1, 18, 5, 0, -1, -1, 34, -1, -1, 19, 5, 0};
static __constant__ float m2l_coef_m1_p5[448] = {
  0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 6.0f, 0.0f, 0.0f, 2.0f, 0.0f, 0.0f, 0.5f, 0.0f, 3.0f, 3.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.5f, 0.0f, 3.0f, 0.0f, 3.0f, 0.0f, 0.0f, 0.0f, 0.5f, 0.0f, 0.0f, 6.0f, 0.0f, 0.0f, 2.0f, 0.0f, 0.5f, 0.0f, 0.0f, 3.0f, 3.0f, 0.0f, 0.0f, 0.0f, 0.5f, 0.0f, 0.0f, 0.0f, 6.0f, 0.0f, 0.0f, 2.0f, 0.5f, 0.0f, 15.0f, 0.0f, 0.0f, 12.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 10.0f, 5.0f, 0.0f, 4.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 10.0f, 0.0f, 5.0f, 4.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 5.0f, 10.0f, 0.0f, 0.0f, 4.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 5.0f, 5.0f, 5.0f, 0.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 5.0f, 0.0f, 10.0f, 0.0f, 0.0f, 4.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 15.0f, 0.0f, 0.0f, 12.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 10.0f, 5.0f, 0.0f, 4.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 5.0f, 10.0f, 0.0f, 0.0f, 4.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 0.0f, 15.0f, 0.0f, 0.0f, 12.0f, 0.3333333432674408f, -9.934107758624577e-09f, 28.0f, 0.0f, 0.0f, 36.0f, 0.0f, 0.0f, 0.25f, 0.0f, 21.0f, 7.0f, 0.0f, 18.0f, 0.0f, 0.0f, 0.25f, 0.0f, 21.0f, 0.0f, 7.0f, 18.0f, 0.0f, 0.0f, 0.25f, 0.0f, 14.0f, 14.0f, 0.0f, 6.0f, 6.0f, 0.0f, 0.25f, 0.0f, 14.0f, 7.0f, 7.0f, 6.0f, 0.0f, 0.0f, 0.25f, 0.0f, 14.0f, 0.0f, 14.0f, 6.0f, 0.0f, 6.0f, 0.25f, 0.0f, 7.0f, 21.0f, 0.0f, 0.0f, 18.0f, 0.0f, 0.25f, 0.0f, 7.0f, 14.0f, 7.0f, 0.0f, 6.0f, 0.0f, 0.25f, 0.0f, 7.0f, 7.0f, 14.0f, 0.0f, 0.0f, 6.0f, 0.25f, 0.0f, 7.0f, 0.0f, 21.0f, 0.0f, 0.0f, 18.0f, 0.25f, 0.0f, 0.0f, 28.0f, 0.0f, 0.0f, 36.0f, 0.0f, 0.25f, 0.0f, 0.0f, 21.0f, 7.0f, 0.0f, 18.0f, 0.0f, 0.25f, 0.0f, 0.0f, 14.0f, 14.0f, 0.0f, 6.0f, 6.0f, 0.25f, 0.0f, 0.0f, 7.0f, 21.0f, 0.0f, 0.0f, 18.0f, 0.25f, 0.0f, 0.0f, 0.0f, 28.0f, 0.0f, 0.0f, 36.0f, 0.25f, 0.0f, 45.0f, 0.0f, 0.0f, 80.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 36.0f, 9.0f, 0.0f, 48.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 36.0f, 0.0f, 9.0f, 48.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 27.0f, 18.0f, 0.0f, 24.0f, 8.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 27.0f, 9.0f, 9.0f, 24.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 27.0f, 0.0f, 18.0f, 24.0f, 0.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 27.0f, 0.0f, 8.0f, 24.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 18.0f, 9.0f, 8.0f, 8.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 9.0f, 18.0f, 8.0f, 0.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 0.0f, 27.0f, 8.0f, 0.0f, 24.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 36.0f, 0.0f, 0.0f, 48.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 27.0f, 9.0f, 0.0f, 24.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 18.0f, 18.0f, 0.0f, 8.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 9.0f, 27.0f, 0.0f, 0.0f, 24.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 0.0f, 36.0f, 0.0f, 0.0f, 48.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 45.0f, 0.0f, 0.0f, 80.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 36.0f, 9.0f, 0.0f, 48.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 27.0f, 18.0f, 0.0f, 24.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 18.0f, 27.0f, 0.0f, 8.0f, 24.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 9.0f, 36.0f, 0.0f, 0.0f, 48.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 0.0f, 45.0f, 0.0f, 0.0f, 80.0f, 0.20000000298023224f, -2.9802322831784522e-09f};
static __constant__ unsigned char m2l_w_m1_p5[406] = {
  1, 4, 5, 6, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 2, 5, 7, 8, 11, 13, 14, 16, 17, 18, 21, 23, 24, 26, 27, 28, 30, 31, 32, 33, 36, 38, 39, 41, 42, 43, 45, 46, 47, 48, 50, 51, 52, 53, 54, 3, 6, 8, 9, 12, 14, 15, 17, 18, 19, 22, 24, 25, 27, 28, 29, 31, 32, 33, 34, 37, 39, 40, 42, 43, 44, 46, 47, 48, 49, 51, 52, 53, 54, 55, 4, 10, 11, 12, 20, 21, 22, 23, 24, 25, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 5, 11, 13, 14, 21, 23, 24, 26, 27, 28, 36, 38, 39, 41, 42, 43, 45, 46, 47, 48, 6, 12, 14, 15, 22, 24, 25, 27, 28, 29, 37, 39, 40, 42, 43, 44, 46, 47, 48, 49, 7, 13, 16, 17, 23, 26, 27, 30, 31, 32, 38, 41, 42, 45, 46, 47, 50, 51, 52, 53, 8, 14, 17, 18, 24, 27, 28, 31, 32, 33, 39, 42, 43, 46, 47, 48, 51, 52, 53, 54, 9, 15, 18, 19, 25, 28, 29, 32, 33, 34, 40, 43, 44, 47, 48, 49, 52, 53, 54, 55, 10, 20, 21, 22, 35, 36, 37, 38, 39, 40, 11, 21, 23, 24, 36, 38, 39, 41, 42, 43, 12, 22, 24, 25, 37, 39, 40, 42, 43, 44, 13, 23, 26, 27, 38, 41, 42, 45, 46, 47, 14, 24, 27, 28, 39, 42, 43, 46, 47, 48, 15, 25, 28, 29, 40, 43, 44, 47, 48, 49, 16, 26, 30, 31, 41, 45, 46, 50, 51, 52, 17, 27, 31, 32, 42, 46, 47, 51, 52, 53, 18, 28, 32, 33, 43, 47, 48, 52, 53, 54, 19, 29, 33, 34, 44, 48, 49, 53, 54, 55, 20, 35, 36, 37, 21, 36, 38, 39, 22, 37, 39, 40, 23, 38, 41, 42, 24, 39, 42, 43, 25, 40, 43, 44, 26, 41, 45, 46, 27, 42, 46, 47, 28, 43, 47, 48, 29, 44, 48, 49, 30, 45, 50, 51, 31, 46, 51, 52, 32, 47, 52, 53, 33, 48, 53, 54, 34, 49, 54, 55, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 50, 51, 52, 53, 54, 55};

// loop-form tables of M2L, source order 1, expansion order 6
static __constant__ short m2l_rec_m1_p6[672] = {
  -1, -1, -1, -1, -1, -1, 0, 0, 0, -1, -1, -1, -1, -1, 1, 0, -1, 0, -1, -1, -1, -1, 1, 0, -1, -1, 0, -1, -1, -1, 1, 0, 1, -1, -1, 0, -1, -1, 2, 0, 2, 1, -1, -1, -1, -1, 2, 0, 3, -1, 1, -1, -1, -1, 2, 0, -1, 2, -1, -1, 0, -1, 2, 0, -1, 3, 2, -1, -1, -1, 2, 0, -1, -1, 3, -1, -1, 0, 2, 0, 4, -1, -1, 1, -1, -1, 3, 0, 5, 4, -1, 2, -1, -1, 3, 0, 6, -1, 4, 3, -1, -1, 3, 0, 7, 5, -1, -1, 1, -1, 3, 0, 8, 6, 5, -1, -1, -1, 3, 0, 9, -1, 6, -1, -1, 1, 3, 0, -1, 7, -1, -1, 2, -1, 3, 0, -1, 8, 7, -1, 3, -1, 3, 0, -1, 9, 8, -1, -1, 2, 3, 0, -1, -1, 9, -1, -1, 3, 3, 0, 10, -1, -1, 4, -1, -1, 4, 0, 11, 10, -1, 5, -1, -1, 4, 0, 12, -1, 10, 6, -1, -1, 4, 0, 13, 11, -1, 7, 4, -1, 4, 0, 14, 12, 11, 8, -1, -1, 4, 0, 15, -1, 12, 9, -1, 4, 4, 0, 16, 13, -1, -1, 5, -1, 4, 0, 17, 14, 13, -1, 6, -1, 4, 0, 18, 15, 14, -1, -1, 5, 4, 0, 19, -1, 15, -1, -1, 6, 4, 0, -1, 16, -1, -1, 7, -1, 4, 0, -1, 17, 16, -1, 8, -1, 4, 0, -1, 18, 17, -1, 9, 7, 4, 0, -1, 19, 18, -1, -1, 8, 4, 0, -1, -1, 19, -1, -1, 9, 4, 0, 20, -1, -1, 10, -1, -1, 5, 0, 21, 20, -1, 11, -1, -1, 5, 0, 22, -1, 20, 12, -1, -1, 5, 0, 23, 21, -1, 13, 10, -1, 5, 0, 24, 22, 21, 14, -1, -1, 5, 0, 25, -1, 22, 15, -1, 10, 5, 0, 26, 23, -1, 16, 11, -1, 5, 0, 27, 24, 23, 17, 12, -1, 5, 0, 28, 25, 24, 18, -1, 11, 5, 0, 29, -1, 25, 19, -1, 12, 5, 0, 30, 26, -1, -1, 13, -1, 5, 0, 31, 27, 26, -1, 14, -1, 5, 0, 32, 28, 27, -1, 15, 13, 5, 0, 33, 29, 28, -1, -1, 14, 5, 0, 34, -1, 29, -1, -1, 15, 5, 0, -1, 30, -1, -1, 16, -1, 5, 0, -1, 31, 30, -1, 17, -1, 5, 0, -1, 32, 31, -1, 18, 16, 5, 0, -1, 33, 32, -1, 19, 17, 5, 0, -1, 34, 33, -1, -1, 18, 5, 0, -1, -1, 34, -1, -1, 19, 5, 0, 35, -1, -1, 20, -1, -1, 6, 0, 36, 35, -1, 21, -1, -1, 6, 0, 37, -1, 35, 22, -1, -1, 6, 0, 38, 36, -1, 23, 20, -1, 6, 0, 39, 37, 36, 24, -1, -1, 6, 0, 40, -1, 37, 25, -1, 20, 6, 0, 41, 38, -1, 26, 21, -1, 6, 0, 42, 39, 38, 27, 22, -1, 6, 0, 43, 40, 39, 28, -1, 21, 6, 0, 44, -1, 40, 29, -1, 22, 6, 0, 45, 41, -1, 30, 23, -1, 6, 0, 46, 42, 41, 31, 24, -1, 6, 0, 47, 43, 42, 32, 25, 23, 6, 0, 48, 44, 43, 33, -1, 24, 6, 0, 49, -1, 44, 34, -1, 25, 6, 0, 50, 45, -1, -1, 26, -1, 6, 0, 51, 46, 45, -1, 27, -1, 6, 0, 52, 47, 46, -1, 28, 26, 6, 0, 53, 48, 47, -1, 29, 27, 6, 0, 54, 49, 48, -1, -1, 28, 6, 0, 55, -1, 49, -1, -1, 29, 6, 0, -1, 50, -1, -1, 30, -1, 6, 0, -1, 51, 50, -1, 31, -1, 6, 0, -1, 52, 51, -1, 32, 30, 6, 0, -1, 53, 52, -1, 33, 31, 6, 0, -1, 54, 53, -1, 34, 32, 6, 0, -1, 55, 54, -1, -1, 33, 6, 0, -1, -1, 55, -1, -1, 34, 6, 0};
static __constant__ float m2l_coef_m1_p6[672] = {
  0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 6.0f, 0.0f, 0.0f, 2.0f, 0.0f, 0.0f, 0.5f, 0.0f, 3.0f, 3.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.5f, 0.0f, 3.0f, 0.0f, 3.0f, 0.0f, 0.0f, 0.0f, 0.5f, 0.0f, 0.0f, 6.0f, 0.0f, 0.0f, 2.0f, 0.0f, 0.5f, 0.0f, 0.0f, 3.0f, 3.0f, 0.0f, 0.0f, 0.0f, 0.5f, 0.0f, 0.0f, 0.0f, 6.0f, 0.0f, 0.0f, 2.0f, 0.5f, 0.0f, 15.0f, 0.0f, 0.0f, 12.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 10.0f, 5.0f, 0.0f, 4.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 10.0f, 0.0f, 5.0f, 4.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 5.0f, 10.0f, 0.0f, 0.0f, 4.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 5.0f, 5.0f, 5.0f, 0.0f, 0.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 5.0f, 0.0f, 10.0f, 0.0f, 0.0f, 4.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 15.0f, 0.0f, 0.0f, 12.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 10.0f, 5.0f, 0.0f, 4.0f, 0.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 5.0f, 10.0f, 0.0f, 0.0f, 4.0f, 0.3333333432674408f, -9.934107758624577e-09f, 0.0f, 0.0f, 15.0f, 0.0f, 0.0f, 12.0f, 0.3333333432674408f, -9.934107758624577e-09f, 28.0f, 0.0f, 0.0f, 36.0f, 0.0f, 0.0f, 0.25f, 0.0f, 21.0f, 7.0f, 0.0f, 18.0f, 0.0f, 0.0f, 0.25f, 0.0f, 21.0f, 0.0f, 7.0f, 18.0f, 0.0f, 0.0f, 0.25f, 0.0f, 14.0f, 14.0f, 0.0f, 6.0f, 6.0f, 0.0f, 0.25f, 0.0f, 14.0f, 7.0f, 7.0f, 6.0f, 0.0f, 0.0f, 0.25f, 0.0f, 14.0f, 0.0f, 14.0f, 6.0f, 0.0f, 6.0f, 0.25f, 0.0f, 7.0f, 21.0f, 0.0f, 0.0f, 18.0f, 0.0f, 0.25f, 0.0f, 7.0f, 14.0f, 7.0f, 0.0f, 6.0f, 0.0f, 0.25f, 0.0f, 7.0f, 7.0f, 14.0f, 0.0f, 0.0f, 6.0f, 0.25f, 0.0f, 7.0f, 0.0f, 21.0f, 0.0f, 0.0f, 18.0f, 0.25f, 0.0f, 0.0f, 28.0f, 0.0f, 0.0f, 36.0f, 0.0f, 0.25f, 0.0f, 0.0f, 21.0f, 7.0f, 0.0f, 18.0f, 0.0f, 0.25f, 0.0f, 0.0f, 14.0f, 14.0f, 0.0f, 6.0f, 6.0f, 0.25f, 0.0f, 0.0f, 7.0f, 21.0f, 0.0f, 0.0f, 18.0f, 0.25f, 0.0f, 0.0f, 0.0f, 28.0f, 0.0f, 0.0f, 36.0f, 0.25f, 0.0f, 45.0f, 0.0f, 0.0f, 80.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 36.0f, 9.0f, 0.0f, 48.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 36.0f, 0.0f, 9.0f, 48.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 27.0f, 18.0f, 0.0f, 24.0f, 8.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 27.0f, 9.0f, 9.0f, 24.0f, 0.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 27.0f, 0.0f, 18.0f, 24.0f, 0.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 27.0f, 0.0f, 8.0f, 24.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 18.0f, 9.0f, 8.0f, 8.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 9.0f, 18.0f, 8.0f, 0.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 18.0f, 0.0f, 27.0f, 8.0f, 0.0f, 24.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 36.0f, 0.0f, 0.0f, 48.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 27.0f, 9.0f, 0.0f, 24.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 18.0f, 18.0f, 0.0f, 8.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 9.0f, 27.0f, 0.0f, 0.0f, 24.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 9.0f, 0.0f, 36.0f, 0.0f, 0.0f, 48.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 45.0f, 0.0f, 0.0f, 80.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 36.0f, 9.0f, 0.0f, 48.0f, 0.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 27.0f, 18.0f, 0.0f, 24.0f, 8.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 18.0f, 27.0f, 0.0f, 8.0f, 24.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 9.0f, 36.0f, 0.0f, 0.0f, 48.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 0.0f, 0.0f, 45.0f, 0.0f, 0.0f, 80.0f, 0.20000000298023224f, -2.9802322831784522e-09f, 66.0f, 0.0f, 0.0f, 150.0f, 0.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 55.0f, 11.0f, 0.0f, 100.0f, 0.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 55.0f, 0.0f, 11.0f, 100.0f, 0.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 44.0f, 22.0f, 0.0f, 60.0f, 10.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 44.0f, 11.0f, 11.0f, 60.0f, 0.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 44.0f, 0.0f, 22.0f, 60.0f, 0.0f, 10.0f, 0.1666666716337204f, -4.967053879312289e-09f, 33.0f, 33.0f, 0.0f, 30.0f, 30.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 33.0f, 22.0f, 11.0f, 30.0f, 10.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 33.0f, 11.0f, 22.0f, 30.0f, 0.0f, 10.0f, 0.1666666716337204f, -4.967053879312289e-09f, 33.0f, 0.0f, 33.0f, 30.0f, 0.0f, 30.0f, 0.1666666716337204f, -4.967053879312289e-09f, 22.0f, 44.0f, 0.0f, 10.0f, 60.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 22.0f, 33.0f, 11.0f, 10.0f, 30.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 22.0f, 22.0f, 22.0f, 10.0f, 10.0f, 10.0f, 0.1666666716337204f, -4.967053879312289e-09f, 22.0f, 11.0f, 33.0f, 10.0f, 0.0f, 30.0f, 0.1666666716337204f, -4.967053879312289e-09f, 22.0f, 0.0f, 44.0f, 10.0f, 0.0f, 60.0f, 0.1666666716337204f, -4.967053879312289e-09f, 11.0f, 55.0f, 0.0f, 0.0f, 100.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 11.0f, 44.0f, 11.0f, 0.0f, 60.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 11.0f, 33.0f, 22.0f, 0.0f, 30.0f, 10.0f, 0.1666666716337204f, -4.967053879312289e-09f, 11.0f, 22.0f, 33.0f, 0.0f, 10.0f, 30.0f, 0.1666666716337204f, -4.967053879312289e-09f, 11.0f, 11.0f, 44.0f, 0.0f, 0.0f, 60.0f, 0.1666666716337204f, -4.967053879312289e-09f, 11.0f, 0.0f, 55.0f, 0.0f, 0.0f, 100.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 66.0f, 0.0f, 0.0f, 150.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 55.0f, 11.0f, 0.0f, 100.0f, 0.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 44.0f, 22.0f, 0.0f, 60.0f, 10.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 33.0f, 33.0f, 0.0f, 30.0f, 30.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 22.0f, 44.0f, 0.0f, 10.0f, 60.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 11.0f, 55.0f, 0.0f, 0.0f, 100.0f, 0.1666666716337204f, -4.967053879312289e-09f, 0.0f, 0.0f, 66.0f, 0.0f, 0.0f, 150.0f, 0.1666666716337204f, -4.967053879312289e-09f};
static __constant__ unsigned char m2l_w_m1_p6[840] = {
  1, 4, 5, 6, 10, 11, 12, 13, 14, 15, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 56, 57, 58, 59, 60, 61, 62, 63, 64, 65, 66, 67, 68, 69, 70, 71, 72, 73, 74, 75, 76, 2, 5, 7, 8, 11, 13, 14, 16, 17, 18, 21, 23, 24, 26, 27, 28, 30, 31, 32, 33, 36, 38, 39, 41, 42, 43, 45, 46, 47, 48, 50, 51, 52, 53, 54, 57, 59, 60, 62, 63, 64, 66, 67, 68, 69, 71, 72, 73, 74, 75, 77, 78, 79, 80, 81, 82, 3, 6, 8, 9, 12, 14, 15, 17, 18, 19, 22, 24, 25, 27, 28, 29, 31, 32, 33, 34, 37, 39, 40, 42, 43, 44, 46, 47, 48, 49, 51, 52, 53, 54, 55, 58, 60, 61, 63, 64, 65, 67, 68, 69, 70, 72, 73, 74, 75, 76, 78, 79, 80, 81, 82, 83, 4, 10, 11, 12, 20, 21, 22, 23, 24, 25, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 56, 57, 58, 59, 60, 61, 62, 63, 64, 65, 66, 67, 68, 69, 70, 5, 11, 13, 14, 21, 23, 24, 26, 27, 28, 36, 38, 39, 41, 42, 43, 45, 46, 47, 48, 57, 59, 60, 62, 63, 64, 66, 67, 68, 69, 71, 72, 73, 74, 75, 6, 12, 14, 15, 22, 24, 25, 27, 28, 29, 37, 39, 40, 42, 43, 44, 46, 47, 48, 49, 58, 60, 61, 63, 64, 65, 67, 68, 69, 70, 72, 73, 74, 75, 76, 7, 13, 16, 17, 23, 26, 27, 30, 31, 32, 38, 41, 42, 45, 46, 47, 50, 51, 52, 53, 59, 62, 63, 66, 67, 68, 71, 72, 73, 74, 77, 78, 79, 80, 81, 8, 14, 17, 18, 24, 27, 28, 31, 32, 33, 39, 42, 43, 46, 47, 48, 51, 52, 53, 54, 60, 63, 64, 67, 68, 69, 72, 73, 74, 75, 78, 79, 80, 81, 82, 9, 15, 18, 19, 25, 28, 29, 32, 33, 34, 40, 43, 44, 47, 48, 49, 52, 53, 54, 55, 61, 64, 65, 68, 69, 70, 73, 74, 75, 76, 79, 80, 81, 82, 83, 10, 20, 21, 22, 35, 36, 37, 38, 39, 40, 56, 57, 58, 59, 60, 61, 62, 63, 64, 65, 11, 21, 23, 24, 36, 38, 39, 41, 42, 43, 57, 59, 60, 62, 63, 64, 66, 67, 68, 69, 12, 22, 24, 25, 37, 39, 40, 42, 43, 44, 58, 60, 61, 63, 64, 65, 67, 68, 69, 70, 13, 23, 26, 27, 38, 41, 42, 45, 46, 47, 59, 62, 63, 66, 67, 68, 71, 72, 73, 74, 14, 24, 27, 28, 39, 42, 43, 46, 47, 48, 60, 63, 64, 67, 68, 69, 72, 73, 74, 75, 15, 25, 28, 29, 40, 43, 44, 47, 48, 49, 61, 64, 65, 68, 69, 70, 73, 74, 75, 76, 16, 26, 30, 31, 41, 45, 46, 50, 51, 52, 62, 66, 67, 71, 72, 73, 77, 78, 79, 80, 17, 27, 31, 32, 42, 46, 47, 51, 52, 53, 63, 67, 68, 72, 73, 74, 78, 79, 80, 81, 18, 28, 32, 33, 43, 47, 48, 52, 53, 54, 64, 68, 69, 73, 74, 75, 79, 80, 81, 82, 19, 29, 33, 34, 44, 48, 49, 53, 54, 55, 65, 69, 70, 74, 75, 76, 80, 81, 82, 83, 20, 35, 36, 37, 56, 57, 58, 59, 60, 61, 21, 36, 38, 39, 57, 59, 60, 62, 63, 64, 22, 37, 39, 40, 58, 60, 61, 63, 64, 65, 23, 38, 41, 42, 59, 62, 63, 66, 67, 68, 24, 39, 42, 43, 60, 63, 64, 67, 68, 69, 25, 40, 43, 44, 61, 64, 65, 68, 69, 70, 26, 41, 45, 46, 62, 66, 67, 71, 72, 73, 27, 42, 46, 47, 63, 67, 68, 72, 73, 74, 28, 43, 47, 48, 64, 68, 69, 73, 74, 75, 29, 44, 48, 49, 65, 69, 70, 74, 75, 76, 30, 45, 50, 51, 66, 71, 72, 77, 78, 79, 31, 46, 51, 52, 67, 72, 73, 78, 79, 80, 32, 47, 52, 53, 68, 73, 74, 79, 80, 81, 33, 48, 53, 54, 69, 74, 75, 80, 81, 82, 34, 49, 54, 55, 70, 75, 76, 81, 82, 83, 35, 56, 57, 58, 36, 57, 59, 60, 37, 58, 60, 61, 38, 59, 62, 63, 39, 60, 63, 64, 40, 61, 64, 65, 41, 62, 66, 67, 42, 63, 67, 68, 43, 64, 68, 69, 44, 65, 69, 70, 45, 66, 71, 72, 46, 67, 72, 73, 47, 68, 73, 74, 48, 69, 74, 75, 49, 70, 75, 76, 50, 71, 77, 78, 51, 72, 78, 79, 52, 73, 79, 80, 53, 74, 80, 81, 54, 75, 81, 82, 55, 76, 82, 83, 56, 57, 58, 59, 60, 61, 62, 63, 64, 65, 66, 67, 68, 69, 70, 71, 72, 73, 74, 75, 76, 77, 78, 79, 80, 81, 82, 83};

#define CPPE_M2L_GENERATED(X) \
  X(1, 5, m2l_m1_p5, 35, 55) \
  X(1, 6, m2l_m1_p6, 56, 83)

#define CPPE_SHIFTS_GENERATED(X) \
  X(1, 5, 35, 55) \
  X(1, 6, 56, 83)

#define CPPE_M2L_TABLES(X) \
  X(1, 5, m1_p5, 56, 35, 55) \
  X(1, 6, m1_p6, 84, 56, 83)
