// isp_fused_spec_u8.cu - the fused kernel specialised for FMT_U8 input (see isp_fused_spec.inl).
#define IMOP_SPEC_FMT FMT_U8
#define IMOP_SPEC_LAUNCH launch_fused_spec_u8
#include "isp_fused_spec.inl"
