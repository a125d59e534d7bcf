// isp_fused_spec_p12.cu - the fused kernel specialised for FMT_P12 input (see isp_fused_spec.inl).
#define IMOP_SPEC_FMT FMT_P12
#define IMOP_SPEC_LAUNCH launch_fused_spec_p12
#include "isp_fused_spec.inl"
