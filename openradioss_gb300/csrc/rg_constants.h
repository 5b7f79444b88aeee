// Generated by gen_constants.py from the reference's constant module
// (common_source/modules/constant_mod.F).  Exact IEEE-754 binary64
// values of the chained parameter expressions; do not edit by hand.
#pragma once

#define RG_ZERO         (0x0.0p+0) /* 0 */
#define RG_ONE          (0x1.0000000000000p+0) /* 1 */
#define RG_TWO          (0x1.0000000000000p+1) /* 2 */
#define RG_THREE        (0x1.8000000000000p+1) /* 3 */
#define RG_FOUR         (0x1.0000000000000p+2) /* 4 */
#define RG_EIGHT        (0x1.0000000000000p+3) /* 8 */
#define RG_TEN          (0x1.4000000000000p+3) /* 10 */
#define RG_HUNDRED      (0x1.9000000000000p+6) /* 100 */
#define RG_HALF         (0x1.0000000000000p-1) /* 0.5 */
#define RG_THIRD        (0x1.5555555555555p-2) /* 0.33333333333333331 */
#define RG_FOURTH       (0x1.0000000000000p-2) /* 0.25 */
#define RG_ONE_OVER_8   (0x1.0000000000000p-3) /* 0.125 */
#define RG_ONE_OVER_64  (0x1.0000000000000p-6) /* 0.015625 */
#define RG_TWO_THIRD    (0x1.5555555555555p-1) /* 0.66666666666666663 */
#define RG_THREE_HALF   (0x1.8000000000000p+0) /* 1.5 */
#define RG_ONEP333      (0x1.553f7ced91687p+0) /* 1.333 */
#define RG_ONEP1        (0x1.199999999999ap+0) /* 1.1000000000000001 */
#define RG_ZEP9         (0x1.ccccccccccccdp-1) /* 0.90000000000000002 */
#define RG_EM01         (0x1.999999999999ap-4) /* 0.10000000000000001 */
#define RG_EM03         (0x1.0624dd2f1a9fcp-10) /* 0.001 */
#define RG_EM06         (0x1.0c6f7a0b5ed8dp-20) /* 9.9999999999999995e-07 */
#define RG_EM10         (0x1.b7cdfd9d7bdbbp-34) /* 1e-10 */
#define RG_EM15         (0x1.203af9ee75616p-50) /* 1.0000000000000001e-15 */
#define RG_EM20         (0x1.79ca10c924223p-67) /* 9.9999999999999995e-21 */
#define RG_EM30         (0x1.4484bfeebc29fp-100) /* 9.9999999999999991e-31 */
#define RG_EP02         (0x1.9000000000000p+6) /* 100 */
#define RG_EP06         (0x1.e848000000000p+19) /* 1000000 */
#define RG_EP20         (0x1.5af1d78b58c40p+66) /* 1e+20 */
#define RG_EP30         (0x1.93e5939a08ceap+99) /* 1e+30 */
#define RG_ZEP499       (0x1.fef9db22d0e57p-2) /* 0.49900000000000005 */
#define RG_FOUR_OVER_3  (0x1.5555555555555p+0) /* 1.3333333333333333 */
#define RG_FIVE         (0x1.4000000000000p+2) /* 5 */
#define RG_SIX          (0x1.8000000000000p+2) /* 6 */
#define RG_TWELVE       (0x1.8000000000000p+3) /* 12 */
#define RG_ONE_OVER_6   (0x1.5555555555555p-3) /* 0.16666666666666666 */
#define RG_ONE_OVER_12  (0x1.5555555555555p-4) /* 0.083333333333333329 */
#define RG_EM04         (0x1.a36e2eb1c432dp-14) /* 0.0001 */
#define RG_EP03         (0x1.f400000000000p+9) /* 1000 */
#define RG_ZEP81        (0x1.9eb851eb851ecp-1) /* 0.81000000000000005 */
#define RG_ZEP072169    (0x1.279aae6c8f756p-4) /* 0.072169000000000011 */
#define RG_ONEP414      (0x1.69fbe76c8b439p+0) /* 1.4139999999999999 */
#define RG_ONE_OVER_9   (0x1.c71c71c71c71cp-4) /* 0.1111111111111111 */
#define RG_THREE_OVER_4 (0x1.8000000000000p-1) /* 0.75 */
#define RG_FOUR_OVER_5  (0x1.999999999999ap-1) /* 0.80000000000000004 */
#define RG_EM07         (0x1.ad7f29abcaf48p-24) /* 9.9999999999999995e-08 */
#define RG_NINE         (0x1.2000000000000p+3) /* 9 */
#define RG_ONEP00001    (0x1.0000a7c5ac472p+0) /* 1.0000100000000001 */
#define RG_SP_1P1       (0x1.19999a0000000p+0) /* 1.1000000238418579: REAL*4 literal 1.1 */
