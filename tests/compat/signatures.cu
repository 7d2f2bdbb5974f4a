// Compiled against the reference's own headers (include/datatypes.h
// configured, include/cuda_extraction.h): every entry point must match the
// declaration in tetragpu_compat.h and resolve from libtetragpu.so at link time.
#include "datatypes.h"
#include "cuda_extraction.h"
#include "tetragpu_compat.h"

int main()
{
    void *volatile p[] = {
        (void *)(void (*)(const TV_Data &))&make_TV_for_GPU,
        (void *)&make_VE_for_GPU, (void *)&make_VF_for_GPU,
        (void *)&make_EV_GPU_return, (void *)&make_EV_GPU,
        (void *)&make_TF_GPU_return, (void *)&make_TF_GPU,
        (void *)&make_TE_GPU_return, (void *)&make_TE_GPU,
        (void *)&make_FV_GPU_return, (void *)&make_FV_GPU,
        (void *)&make_FE_GPU_return, (void *)&make_FE_GPU,
        (void *)&get_approx_max_VV,
        (void *)&make_VV_GPU_return, (void *)&make_VV_GPU,
        (void *)(device_VT * (*)(const TV_Data &))&make_VT_GPU_return,
        (void *)(device_VT * (*)(const VT_Data &))&make_VT_GPU_return,
    };
    return p[0] == nullptr;
}
