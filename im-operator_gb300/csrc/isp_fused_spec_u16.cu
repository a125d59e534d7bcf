// isp_fused_spec_u16.cu - the fused kernel specialised for FMT_U16 input (see isp_fused_spec.inl).
#define IMOP_SPEC_FMT FMT_U16
#define IMOP_SPEC_LAUNCH launch_fused_spec_u16
#include "isp_fused_spec.inl"
