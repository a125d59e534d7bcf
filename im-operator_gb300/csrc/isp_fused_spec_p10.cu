// isp_fused_spec_p10.cu - the fused kernel specialised for FMT_P10 input (see isp_fused_spec.inl).
#define IMOP_SPEC_FMT FMT_P10
#define IMOP_SPEC_LAUNCH launch_fused_spec_p10
#include "isp_fused_spec.inl"
