// EULER kernels (reference: Euler1D_SweptShared.cu:183-746), float and double instances.
#include "engine.cuh"
#include "persistent.cuh"

namespace sw {
namespace {
template <typename T>
Ops make_ops() {
    using Sc = Scheme<SW_EULER, T>;
    Ops o{};
    o.problem = SW_EULER;
    o.prec = (int)sizeof(T);
    o.R = Sc::R;
    o.S = Sc::S;
    o.C = 3;
    o.cell = sizeof(typename Sc::G);
    o.max_threads = Sc::MAXT;
    o.classic = launch_classic<SW_EULER, T>;
    o.swept = launch_swept<SW_EULER, T>;
    o.persistent = launch_persistent<SW_EULER, T>;
    o.pack = launch_pack<T>;
    o.unpack = launch_unpack<T>;
    o.swept_smem = smem_of<SW_EULER, T>;
    o.batch_swept = launch_swept_batch<SW_EULER, T>;
    o.batch_classic = launch_classic_batch<SW_EULER, T>;
    o.batch_persistent = launch_persistent_batch<SW_EULER, T>;
    return o;
}
}  // namespace

const Ops *euler_ops(int prec) {
    static const Ops f = make_ops<float>();
    static const Ops d = make_ops<double>();
    return prec == 4 ? &f : (prec == 8 ? &d : nullptr);
}
}  // namespace sw
