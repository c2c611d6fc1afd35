/*
 * wavey_status.h -- status codes shared by libwavey_cuda.so and
 * libwavey_host.so.
 *
 * The reference backend returns Result<Option<Spectra>, String>
 * (core/wavey-solver/src/gpu_fdtd.rs:45-54): Ok(Some) = done, Ok(None) =
 * cancelled, Err = a limit or device failure.  Over the C-ABI that becomes
 * WAVEY_OK, WAVEY_CANCELLED and a negative code, with the message available
 * from wavey_cuda_last_error().
 */
#ifndef WAVEY_STATUS_H
#define WAVEY_STATUS_H

#define WAVEY_OK 0
#define WAVEY_CANCELLED 1
#define WAVEY_E_INVALID (-1)  /* a bad argument: null pointer, index out of range, ... */
#define WAVEY_E_LIMIT (-2)    /* a size limit: cells, steps, boundary nodes, memory */
#define WAVEY_E_CUDA (-3)     /* a CUDA runtime or driver error */
#define WAVEY_E_NOMEM (-4)    /* a host or device allocation failed */
#define WAVEY_E_DEVICE (-5)   /* the kernel reported an error word (bounded wait ran out, bad index) */

#endif
