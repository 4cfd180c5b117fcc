// cnns_t3.cu -- the component search kernel for 3D points, every launch shape.
#include "cnns_search.cuh"

namespace emst {

cudaError_t launch_cnns_t3(const CnnsArgs& a, bool clouds, int shape, int sms, cudaStream_t s)
{
    return clouds ? launch_dim<3, true>(a, shape, sms, s) : launch_dim<3, false>(a, shape, sms, s);
}

cudaError_t launch_knn_first3(const CnnsArgs& a, bool clouds, bool learned, uint64_t* klist, unsigned char* kcur,
                             const uint32_t* iperm, int sms, cudaStream_t s)
{
    if (learned) return launch_knn<3, false, true>(a, klist, kcur, iperm, sms, s);  // single clouds only
    return clouds ? launch_knn<3, true, false>(a, klist, kcur, iperm, sms, s)
                  : launch_knn<3, false, false>(a, klist, kcur, iperm, sms, s);
}

}  // namespace emst
