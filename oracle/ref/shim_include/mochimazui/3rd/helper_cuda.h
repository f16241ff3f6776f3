// Empty stand-in for the reference's vendored helper_cuda.h (not shipped in
// the reference tree); only its include is needed by ras_define.h.
#pragma once
