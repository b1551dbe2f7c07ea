/* Device models built outside the library (CUDA C++; the counterpart of the reference's
 * model source handed to ocl_add_source, tay/ocl.c:274-282).
 *
 * A host that needs a see / act pair the library does not ship writes it as CUDA policies
 * against this header, compiles it into its own shared library for sm_103a, and registers
 * it with tgpu_register_model_library (or tgpu_register_model) from include/tay_gpu.h.
 * Its func names then select it in tay_add_see / tay_add_act on TAY_GPU_Z_GRID groups.
 *
 * Build (the recipe tay_gb300._build.build_model runs):
 *   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 --expt-relaxed-constexpr \
 *        -Xcompiler -fPIC -shared --cudart shared \
 *        -I include -I tay_gb300/csrc/gpu my_model.cu -o libmy_model.so
 *
 * What a model provides (tay_gb300/csrc/gpu/model_boids.cu is a complete example):
 *   - a record codec: kAgentBytes (the AoS record size: 8-byte tag, float4 position at +8,
 *     then the model's fields), pack (record words -> the model's SoA streams) and unpack
 *     (streams -> record words, per program);
 *   - per see kernel a pass policy P with SeeCtx / ActCtx / Seer types, kSeenF4 and
 *     seen_stream (the float4 streams read from seen agents; stream 0 is the position),
 *     load (the seer's state before its walk), see (one seen agent that passed the box
 *     test; may run on any of the library's walks, so it must not depend on the visiting
 *     order beyond float rounding), finish (the seer's results, plus a fused act);
 *   - per standalone act kernel a policy A with ActCtx and act;
 *   - tgpu::KernelDesc entries (launch_see_t<P> / launch_act_t<A>, prepare_see_t<P>) and
 *     tgpu::ProgramDesc entries (the pass sequences the model runs), gathered in a
 *     tgpu::ModelDesc whose name and func names no other model uses;
 *   - extern "C" const void *tgpu_model_entry(unsigned *abi): stores TGPU_MODEL_ABI and
 *     returns the descriptor (which must live as long as the process).
 * The seen agents' fields are read only; a seer writes only its own streams, so there are
 * no atomics on agent state (the reference's rule, README.md:64).
 */
#ifndef TAY_GPU_MODEL_CUH
#define TAY_GPU_MODEL_CUH

#include "model.cuh"
#include "tay_gpu.h"

/* The model interface's layout stamp as this translation unit sees it. */
#define TGPU_MODEL_ABI (::tgpu::kModelAbi)

#endif
