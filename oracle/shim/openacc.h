/* Host-only stand-in for the OpenACC runtime calls made by the reference
 * solvers (oracle test infrastructure only).  Compiled without -fopenacc the
 * reference's `#pragma acc` regions run serially on the host. */
#pragma once
typedef enum { acc_device_none = 0, acc_device_host = 2, acc_device_nvidia = 4 } acc_device_t;
inline int acc_get_num_devices(acc_device_t) { return 1; }
inline void acc_set_device_num(int, acc_device_t) {}
inline int acc_get_device_num(acc_device_t) { return 0; }
