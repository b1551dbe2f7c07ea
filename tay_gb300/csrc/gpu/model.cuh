// Device model registry: the GB300 counterpart of the reference's "func_name + model
// source pasted into an OpenCL program" mechanism (tay/ocl.c:100-177, 274-291).
//
// A model is a set of __device__ see/act functions compiled into the library.  It is
// found by the func_name strings the host passes to tay_add_see / tay_add_act, exactly
// the names the reference's OpenCL path keys its generated kernels on
// (tay/ocl.c:284-291).  For every pass sequence the model supports, it provides kernels
// in which an act pass that directly follows a see pass of the same group is fused into
// the see kernel's epilogue.
#pragma once

#include "see.cuh"

namespace tgpu {

enum StreamRole : uint8_t {
    kState = 0,  // persistent, reordered by every sort
    kStep = 1,   // valid within one step only, written before it is read
};

// One kernel of a model's step program: a see pass (optionally with the following act
// fused in) or a standalone act pass.
struct KernelDesc {
    const char *see;                   // see func name, or nullptr for an act-only kernel
    const char *act;                   // act func name (fused when see != nullptr), or nullptr
    uint32_t writes_f4;                // float4 streams the kernel writes
    uint32_t writes_u32;               // u32 streams the kernel writes
    uint32_t seen_f4;                  // float4 streams read from other agents (staged)
    int staged_f4;                     // number of staged float4 streams per agent
    // launch with the descriptor filled by the runtime
    // returns true when it stored the records through L.wt (the pass declares a Codec)
    bool (*launch_see)(const SeeLaunch &L, size_t smem, cudaStream_t st);
    void (*launch_act)(const ActLaunch &L, cudaStream_t st);
    cudaError_t (*prepare)(size_t smem);  // raises the kernel's dynamic shared memory limit
    int accumulates;                   // see kernel adds onto the seer's stored fields (several see
                                       // passes of one group accumulate); 0: starts from zero
    int pair_list;                     // 1: can record a pair list for the next see pass (P::keep);
                                       // 2: can replay the previous pass's list (P::replay_ok)
};

// A supported pass sequence: the func names in registration order, and the kernels
// that run it.
struct ProgramDesc {
    int passes;
    const char *names[4];
    int kernels;
    int kernel_index[4];  // into ModelDesc::kernels
};

struct ModelDesc {
    const char *name;
    uint32_t agent_bytes;
    int nf4, nu32;
    uint8_t role_f4[kMaxF4];
    uint8_t role_u32[kMaxU32];
    uint32_t see_ctx_bytes;   // bytes of the device see context (host context is copied in)
    uint32_t act_ctx_bytes;
    const KernelDesc *kernels;
    int nkernels;
    const ProgramDesc *programs;
    int nprograms;
    // AoS -> SoA; the packed positions' extent is reduced into *extent (reset by the caller)
    void (*pack)(const uint32_t *aos, uint32_t n, const PassIO &io, BoxAcc *extent, cudaStream_t st);
    void (*unpack)(uint32_t *aos, uint32_t n, const PassIO &io, uint32_t program, cudaStream_t st);
    int nonpoint;  // 1: box agents, float4 stream 0 the min corner (the position), 1 the max
};

// Layout stamp of the model interface: a model compiled against other definitions of the
// launch descriptors, of the segment spec they point to or of ModelDesc carries another
// value and is refused at registration.
constexpr unsigned kModelAbi = 0x01000001u ^ ((unsigned)sizeof(SeeLaunch) << 12) ^ ((unsigned)sizeof(ActLaunch) << 4) ^
                               (unsigned)sizeof(ModelDesc) ^ ((unsigned)sizeof(KernelDesc) << 20) ^
                               ((unsigned)sizeof(ProgramDesc) << 8) ^ ((unsigned)sizeof(SegmentSpec) << 24);

// The SPH model's adjoint kernels (used by adjoint.cu).
struct SphAdjointKernels {
    bool (*force_record)(const SeeLaunch &L, size_t smem, cudaStream_t st);  // force + integrate, also stores a
    cudaError_t (*force_record_prepare)(size_t smem);
    void (*integrate_adj)(const ActLaunch &L, cudaStream_t st);
    bool (*force_adj)(const SeeLaunch &L, size_t smem, cudaStream_t st);  // walks, records the pair list
    cudaError_t (*force_adj_prepare)(size_t smem);
    bool (*force_adj_replay)(const SeeLaunch &L, size_t smem, cudaStream_t st);  // replays a stored list
    cudaError_t (*force_adj_replay_prepare)(size_t smem);
    bool (*density_adj)(const SeeLaunch &L, size_t smem, cudaStream_t st);
    cudaError_t (*density_adj_prepare)(size_t smem);
    void (*scatter_adj)(const ActLaunch &L, cudaStream_t st);
    uint32_t ctx_bytes;
};
const SphAdjointKernels *sph_adjoint_kernels();

const ModelDesc *model_test_basic();
const ModelDesc *model_boids();
const ModelDesc *model_sph();
const ModelDesc *model_box();

// helpers used by the model translation units
template <class P>
bool launch_see_t(const SeeLaunch &L, size_t smem, cudaStream_t st) {
    if (!L.ctas) return L.wt != nullptr;  // nothing to write
    // the row kernel with the warp-union and hit-mask walks only when a tuning asks for them
    const bool warp_walks = L.hit_masks || L.union_factor > 1;
    if constexpr (!std::is_void_v<typename see_detail::CodecOf<P>::type>) {
        // write-through launch (the last pass of a run): the walk without row staging
        if (L.wt) {
            if (L.rows && warp_walks)
                see_rows_kernel<P, false, true, true><<<L.ctas, kSeeThreads, 0, st>>>(L);
            else if (L.rows)
                see_rows_kernel<P, false, true, false><<<L.ctas, kSeeThreads, 0, st>>>(L);
            else
                see_kernel<P, true><<<L.ctas, kSeeThreads, smem, st>>>(L);
            return true;
        }
    }
    if (L.rows && L.stage_cap)
        see_rows_kernel<P, true><<<L.ctas, kSeeThreads, smem, st>>>(L);
    else if (L.rows && warp_walks)
        see_rows_kernel<P><<<L.ctas, kSeeThreads, 0, st>>>(L);
    else if (L.rows)
        see_rows_kernel<P, false, false, false><<<L.ctas, kSeeThreads, 0, st>>>(L);
    else
        see_kernel<P><<<L.ctas, kSeeThreads, smem, st>>>(L);
    return false;
}
template <class A>
void launch_act_t(const ActLaunch &L, cudaStream_t st) {
    if (L.tiles) act_kernel<A><<<L.tiles, kSortThreads, 0, st>>>(L);
}
template <class P>
cudaError_t prepare_see_t(size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(see_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if constexpr (!std::is_void_v<typename see_detail::CodecOf<P>::type>) {
        e = cudaFuncSetAttribute(see_kernel<P, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaFuncSetAttribute(see_rows_kernel<P, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
template <class M>
void pack_t(const uint32_t *aos, uint32_t n, const PassIO &io, BoxAcc *extent, cudaStream_t st) {
    if (n) pack_kernel<M><<<(n + 255) / 256, 256, 0, st>>>(aos, n, io, extent);
}
template <class M>
void unpack_t(uint32_t *aos, uint32_t n, const PassIO &io, uint32_t program, cudaStream_t st) {
    if (n) unpack_kernel<M><<<(n + 255) / 256, 256, 0, st>>>(aos, n, io, program);
}

TGPU_D float4 ld_words4(const uint32_t *w) {
    return make_float4(__uint_as_float(w[0]), __uint_as_float(w[1]), __uint_as_float(w[2]), __uint_as_float(w[3]));
}
TGPU_D void st_words4(uint32_t *w, const float4 &v) {
    w[0] = __float_as_uint(v.x);
    w[1] = __float_as_uint(v.y);
    w[2] = __float_as_uint(v.z);
    w[3] = __float_as_uint(v.w);
}

}  // namespace tgpu
