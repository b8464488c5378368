// KS kernels (reference: KS1D_SweptShared.cu:111-394), float and double instances.
#include "engine.cuh"
#include "persistent.cuh"

namespace sw {
namespace {
template <typename T>
Ops make_ops() {
    using Sc = Scheme<SW_KS, T>;
    Ops o{};
    o.problem = SW_KS;
    o.prec = (int)sizeof(T);
    o.R = Sc::R;
    o.S = Sc::S;
    o.C = 1;
    o.cell = sizeof(typename Sc::G);
    o.max_threads = Sc::MAXT;
    o.classic = launch_classic<SW_KS, T>;
    o.swept = launch_swept<SW_KS, T>;
    o.persistent = launch_persistent<SW_KS, T>;
    o.pack = nullptr;
    o.unpack = nullptr;
    o.swept_smem = smem_of<SW_KS, T>;
    o.batch_swept = launch_swept_batch<SW_KS, T>;
    o.batch_classic = launch_classic_batch<SW_KS, T>;
    o.batch_persistent = launch_persistent_batch<SW_KS, T>;
    return o;
}
}  // namespace

#ifdef SW_KS_DIVIDE_TU
const Ops *ks_divide_ops(int prec) {
#else
const Ops *ks_ops(int prec) {
#endif
    static const Ops f = make_ops<float>();
    static const Ops d = make_ops<double>();
    return prec == 4 ? &f : (prec == 8 ? &d : nullptr);
}
}  // namespace sw
