/* Host-only stand-in for the OpenACC runtime header.
 *
 * Test infrastructure: lets the reference's C++ sources (which include
 * "openacc.h" and call a handful of runtime functions) compile with plain g++
 * as a single-device serial program.  Every OpenACC pragma is ignored by g++,
 * so each `#pragma acc parallel loop` becomes an ordinary serial loop.
 * Functions provided are the only ones the reference calls:
 * acc_get_num_devices, acc_get_device_type, acc_set_device_num, acc_wait_all,
 * acc_async_wait_all. */
#ifndef IBTFO_ORACLE_OPENACC_STANDIN_H
#define IBTFO_ORACLE_OPENACC_STANDIN_H
typedef int acc_device_t;
enum { acc_device_default = 0 };
static inline acc_device_t acc_get_device_type(void) { return acc_device_default; }
static inline int acc_get_num_devices(acc_device_t) { return 1; }
static inline void acc_set_device_num(int, acc_device_t) {}
static inline void acc_wait_all(void) {}
static inline void acc_async_wait_all(void) {}
#endif
