// asg_knn_net.cuh -- generated by gen_knn_net.py; do not edit.
// Comparator networks of k_knn_t33's queue flush (checked by the 0-1
// principle in the generator).  A comparator leaves min in x, max in y.
#pragma once

namespace asg {

constexpr int KNN_QUEUE = 16;

#define ASG_CX(x, y) { const float lo_ = fminf(x, y); y = fmaxf(x, y); x = lo_; }

// Batcher's odd-even merge sort of v[0..15] ascending (63 comparators)
__device__ __forceinline__ void knn_sort16(float (&v)[16])
{
    ASG_CX(v[0], v[1])
    ASG_CX(v[2], v[3])
    ASG_CX(v[0], v[2])
    ASG_CX(v[1], v[3])
    ASG_CX(v[1], v[2])
    ASG_CX(v[4], v[5])
    ASG_CX(v[6], v[7])
    ASG_CX(v[4], v[6])
    ASG_CX(v[5], v[7])
    ASG_CX(v[5], v[6])
    ASG_CX(v[0], v[4])
    ASG_CX(v[2], v[6])
    ASG_CX(v[2], v[4])
    ASG_CX(v[1], v[5])
    ASG_CX(v[3], v[7])
    ASG_CX(v[3], v[5])
    ASG_CX(v[1], v[2])
    ASG_CX(v[3], v[4])
    ASG_CX(v[5], v[6])
    ASG_CX(v[8], v[9])
    ASG_CX(v[10], v[11])
    ASG_CX(v[8], v[10])
    ASG_CX(v[9], v[11])
    ASG_CX(v[9], v[10])
    ASG_CX(v[12], v[13])
    ASG_CX(v[14], v[15])
    ASG_CX(v[12], v[14])
    ASG_CX(v[13], v[15])
    ASG_CX(v[13], v[14])
    ASG_CX(v[8], v[12])
    ASG_CX(v[10], v[14])
    ASG_CX(v[10], v[12])
    ASG_CX(v[9], v[13])
    ASG_CX(v[11], v[15])
    ASG_CX(v[11], v[13])
    ASG_CX(v[9], v[10])
    ASG_CX(v[11], v[12])
    ASG_CX(v[13], v[14])
    ASG_CX(v[0], v[8])
    ASG_CX(v[4], v[12])
    ASG_CX(v[4], v[8])
    ASG_CX(v[2], v[10])
    ASG_CX(v[6], v[14])
    ASG_CX(v[6], v[10])
    ASG_CX(v[2], v[4])
    ASG_CX(v[6], v[8])
    ASG_CX(v[10], v[12])
    ASG_CX(v[1], v[9])
    ASG_CX(v[5], v[13])
    ASG_CX(v[5], v[9])
    ASG_CX(v[3], v[11])
    ASG_CX(v[7], v[15])
    ASG_CX(v[7], v[11])
    ASG_CX(v[3], v[5])
    ASG_CX(v[7], v[9])
    ASG_CX(v[11], v[13])
    ASG_CX(v[1], v[2])
    ASG_CX(v[3], v[4])
    ASG_CX(v[5], v[6])
    ASG_CX(v[7], v[8])
    ASG_CX(v[9], v[10])
    ASG_CX(v[11], v[12])
    ASG_CX(v[13], v[14])
}

// a[0..32] and v[0..15] ascending -> a = the 33 smallest of both,
// ascending; returns the 34th smallest.  Batcher's odd-even merge for
// lengths 33 and 16, pruned to the first 34 outputs (101 comparators).
__device__ __forceinline__ float knn_merge33(float (&a)[33], const float (&v)[16])
{
    float w0 = a[0], w1 = a[1], w2 = a[2], w3 = a[3], w4 = a[4], w5 = a[5], w6 = a[6], w7 = a[7], w8 = a[8], w9 = a[9], w10 = a[10], w11 = a[11], w12 = a[12], w13 = a[13], w14 = a[14], w15 = a[15], w16 = a[16], w17 = a[17], w18 = a[18], w19 = a[19], w20 = a[20], w21 = a[21], w22 = a[22], w23 = a[23], w24 = a[24], w25 = a[25], w26 = a[26], w27 = a[27], w28 = a[28], w29 = a[29], w30 = a[30], w31 = a[31], w32 = a[32];
    float w33 = v[0], w34 = v[1], w35 = v[2], w36 = v[3], w37 = v[4], w38 = v[5], w39 = v[6], w40 = v[7], w41 = v[8], w42 = v[9], w43 = v[10], w44 = v[11], w45 = v[12], w46 = v[13], w47 = v[14], w48 = v[15];
    ASG_CX(w0, w33)
    ASG_CX(w32, w33)
    ASG_CX(w16, w32)
    ASG_CX(w8, w41)
    ASG_CX(w24, w41)
    ASG_CX(w8, w16)
    ASG_CX(w24, w32)
    ASG_CX(w41, w33)
    ASG_CX(w4, w37)
    ASG_CX(w20, w37)
    ASG_CX(w12, w45)
    ASG_CX(w28, w45)
    ASG_CX(w12, w20)
    ASG_CX(w28, w37)
    ASG_CX(w4, w8)
    ASG_CX(w12, w16)
    ASG_CX(w20, w24)
    ASG_CX(w28, w32)
    ASG_CX(w37, w41)
    ASG_CX(w2, w35)
    ASG_CX(w18, w35)
    ASG_CX(w10, w43)
    ASG_CX(w26, w43)
    ASG_CX(w10, w18)
    ASG_CX(w26, w35)
    ASG_CX(w6, w39)
    ASG_CX(w22, w39)
    ASG_CX(w14, w47)
    ASG_CX(w30, w47)
    ASG_CX(w14, w22)
    ASG_CX(w30, w39)
    ASG_CX(w6, w10)
    ASG_CX(w14, w18)
    ASG_CX(w22, w26)
    ASG_CX(w30, w35)
    ASG_CX(w2, w4)
    ASG_CX(w6, w8)
    ASG_CX(w10, w12)
    ASG_CX(w14, w16)
    ASG_CX(w18, w20)
    ASG_CX(w22, w24)
    ASG_CX(w26, w28)
    ASG_CX(w30, w32)
    ASG_CX(w35, w37)
    ASG_CX(w1, w34)
    ASG_CX(w17, w34)
    ASG_CX(w9, w42)
    ASG_CX(w25, w42)
    ASG_CX(w9, w17)
    ASG_CX(w25, w34)
    ASG_CX(w5, w38)
    ASG_CX(w21, w38)
    ASG_CX(w13, w46)
    ASG_CX(w29, w46)
    ASG_CX(w13, w21)
    ASG_CX(w29, w38)
    ASG_CX(w5, w9)
    ASG_CX(w13, w17)
    ASG_CX(w21, w25)
    ASG_CX(w29, w34)
    ASG_CX(w3, w36)
    ASG_CX(w19, w36)
    ASG_CX(w11, w44)
    ASG_CX(w27, w44)
    ASG_CX(w11, w19)
    ASG_CX(w27, w36)
    ASG_CX(w7, w40)
    ASG_CX(w23, w40)
    ASG_CX(w15, w48)
    ASG_CX(w31, w48)
    ASG_CX(w15, w23)
    ASG_CX(w31, w40)
    ASG_CX(w7, w11)
    ASG_CX(w15, w19)
    ASG_CX(w23, w27)
    ASG_CX(w31, w36)
    ASG_CX(w3, w5)
    ASG_CX(w7, w9)
    ASG_CX(w11, w13)
    ASG_CX(w15, w17)
    ASG_CX(w19, w21)
    ASG_CX(w23, w25)
    ASG_CX(w27, w29)
    ASG_CX(w31, w34)
    ASG_CX(w1, w2)
    ASG_CX(w3, w4)
    ASG_CX(w5, w6)
    ASG_CX(w7, w8)
    ASG_CX(w9, w10)
    ASG_CX(w11, w12)
    ASG_CX(w13, w14)
    ASG_CX(w15, w16)
    ASG_CX(w17, w18)
    ASG_CX(w19, w20)
    ASG_CX(w21, w22)
    ASG_CX(w23, w24)
    ASG_CX(w25, w26)
    ASG_CX(w27, w28)
    ASG_CX(w29, w30)
    ASG_CX(w31, w32)
    ASG_CX(w34, w35)
    a[0] = w0;
    a[1] = w1;
    a[2] = w2;
    a[3] = w3;
    a[4] = w4;
    a[5] = w5;
    a[6] = w6;
    a[7] = w7;
    a[8] = w8;
    a[9] = w9;
    a[10] = w10;
    a[11] = w11;
    a[12] = w12;
    a[13] = w13;
    a[14] = w14;
    a[15] = w15;
    a[16] = w16;
    a[17] = w17;
    a[18] = w18;
    a[19] = w19;
    a[20] = w20;
    a[21] = w21;
    a[22] = w22;
    a[23] = w23;
    a[24] = w24;
    a[25] = w25;
    a[26] = w26;
    a[27] = w27;
    a[28] = w28;
    a[29] = w29;
    a[30] = w30;
    a[31] = w31;
    a[32] = w32;
    return w34;
}

#undef ASG_CX

}  // namespace asg
