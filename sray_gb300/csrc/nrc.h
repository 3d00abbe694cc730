/* nrc.h -- the radiance cache as the renderer drives it (nrc.cu). */
#ifndef SRAY_NRC_H_
#define SRAY_NRC_H_

#include <stdint.h>
#include <cuda_runtime.h>

namespace sray {

/* allocate and, the first time, initialise the network from `seed` */
int nrc_ensure_ready(uint64_t seed, cudaStream_t s);
/* y[n][3] = network(x[n][9]); x = position scaled to the scene box, normal,
 * direction (the encoding's argument reduction holds for |x| <= 4096) */
int nrc_infer(int n, const float *x, float *y, cudaStream_t s);
/* the renderer's queries: acc[slot] += w.rgb * max(network(x[i]), 0) for
 * i < *count (at most cap), slot = the int in w[i].w */
int nrc_query(const int *count, int cap, const float *x, const float4 *w, float4 *acc, cudaStream_t s);
/* one Adam step on the batch (x[n][9], targets t[n][3]): NRC_TRAIN_KERNELS launches */
#define NRC_TRAIN_KERNELS 9
int nrc_train(int n, const float *x, const float *t, float lr, cudaStream_t s);
/* `steps` Adam steps over consecutive batches of `per` samples of (x, t),
 * replayed from a CUDA graph while the arguments stay the same */
int nrc_train_steps(int steps, int per, const float *x, const float *t, float lr, cudaStream_t s);
/* SRAY_EDEVICE (and the error word cleared) when a tensor-core forward's
 * bounded wait ran out since the last call; waits for stream s */
int nrc_device_error(cudaStream_t s);
/* device address of the last batch's loss */
float *nrc_loss_ptr();
const char *nrc_error();

}  // namespace sray

#endif
