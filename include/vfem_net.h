/*
 * vfem_net.h -- C ABI of the learned part of libvfem: a small BF16 3-D U-Net on
 * the node grid that predicts displacements from (occupancy, modulus, fixed
 * mask, load).  No counterpart in the reference (VulkanFEM has no learned
 * component); the network warm-starts the MG-PCG solve and serves as a learned
 * coarse correction inside flexible CG.  Trained and evaluated with the
 * library's own kernels (vulkanfem_gb300/csrc/unet.cu).
 *
 * Grid: n^3 nodes, n a multiple of 8 (the solver's node grid padded with
 * zeros).  Features: [n^3][16] FP32, channels-last, x fastest; targets
 * [n^3][3]; masks [n^3] (1 = node counted in the loss).  Parameters are one
 * packed FP32 array (per layer: weights [27][Cin][Cout], then bias [Cout]).
 */
#ifndef VFEM_NET_H
#define VFEM_NET_H

#include <stdint.h>

#include "vfem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vfem_net vfem_net;

vfem_status vfem_net_create(int32_t n, vfem_net** out);
void vfem_net_destroy(vfem_net* net);
int64_t vfem_net_num_params(const vfem_net* net);
vfem_status vfem_net_set_params(vfem_net* net, const float* params);
vfem_status vfem_net_get_params(vfem_net* net, float* params);

/* Inference: input [n^3][16] -> output [n^3][3]. */
vfem_status vfem_net_forward(vfem_net* net, const float* input, float* output);

/* Forward + backward over `batch` samples (inputs [batch][n^3][16], targets
 * [batch][n^3][3], masks [batch][n^3]); mean masked-MSE loss to *loss_out;
 * batch-mean gradients to grads (host, num_params floats) when not NULL; one
 * Adam step (beta 0.9/0.999) with learning rate lr when lr > 0. */
vfem_status vfem_net_train_batch(vfem_net* net, const float* inputs, const float* targets, const float* masks,
                                 int32_t batch, float lr, float* grads, float* loss_out);

const char* vfem_net_last_error_message(void);

#ifdef __cplusplus
}
#endif

#endif /* VFEM_NET_H */
