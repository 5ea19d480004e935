/* gpu_phs_transfer.h -- the device handoff of the last Whizard call, C++ linkage.
 *
 * Replaces transfer_to_whizard.h:1-3 of the reference, which declares these three
 * functions without extern "C" (their definitions in phs.cu:1638-1644 are C++), so code
 * written against that header links against this library unchanged.  All three refer to
 * the last c_whizard_gen_phs_from_x_gpu call and return device memory that the library
 * owns until the next call, c_whizard_reset_generator or c_whizard_finalize_gpu_phs; null
 * before the first call or on error (phs_last_error says why).
 */
#ifndef GPU_PHS_TRANSFER_H
#define GPU_PHS_TRANSFER_H

#ifdef __cplusplus
/* Momenta in the reference's sparse layout, [event][2^(n_in + n_out) - 1][4] doubles at
 * slot code - 1 (phs.cu:1364-1373): outgoing particles (codes 2^k) in the lab frame; every
 * code that is an internal branch of some channel holds the sum of its particles'
 * momenta in the centre-of-mass frame, as the reference's buffer ends up after its
 * inverse-map loop (phs.cu:1262-1283, lab boost of the outgoing codes only, phs.cu:1286-1301);
 * other slots 0.  Built on the first request after a call (one kernel, then a device
 * synchronisation).  Replaces get_momentum_device_pointer, phs.cu:1638-1640.  The dense
 * [event][n_out][4] momenta are phs_whizard_momentum_device_pointer (gpu_phs.h). */
double *get_momentum_device_pointer();

/* The beam energies [E1[0..n); E2[0..n)] of the last call.  Replaces
 * get_in_momentum_device_pointer, phs.cu:1642-1644 (prt_in_d, phs.cu:1360-1363). */
double *get_in_momentum_device_pointer();

/* The ok flags [n] of the last call (one byte each, 0 or 1).  Declared in the reference's
 * transfer_to_whizard.h:3 but not defined there. */
bool *get_ok_device_pointer();
#endif

#endif
