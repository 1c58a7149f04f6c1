/* vg_rtc_types.h -- the fixed-width integer types for device code compiled
 * at run time by NVRTC, which has no C library headers. */
#ifndef VG_RTC_TYPES_H
#define VG_RTC_TYPES_H
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef short int16_t;
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
typedef unsigned long long uintptr_t;
#endif
