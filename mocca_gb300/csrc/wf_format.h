// wf_format.h -- the in-memory form of a version-1 MOCCa wavefunction file
// (include/mocca_wf.h), shared by the file layer (wf_format.cpp) and the
// device-context bridge (wf_ctx.cu).
#pragma once

#include <string>
#include <vector>

#include "../../include/mocca_wf.h"

struct mg_wf {
    mg_wf_header h{};
    // one vector per MG_WF_* field; fields with int elements use ints
    std::vector<double> d[MG_WF_NFIELDS];
    std::vector<int> i[MG_WF_NFIELDS];
};

namespace mg {

// true when the field's elements are ints
bool wf_field_is_int(int field);
// shapes that follow from nwt and the symmetries
void wf_derive_shapes(mg_wf_header& h);
// the element count a field must have under the header's shapes
long long wf_field_count(const mg_wf_header& h, int field);
// allocate every field at its count, zeroed
void wf_allocate(mg_wf& w);

}  // namespace mg
