// Link stubs for the reference harness -- TEST INFRASTRUCTURE.
// levelset/levelsetmapper.cpp (the isoparametric QuaQua mapper) does not
// compile as shipped; surfactant/ifacetransp.cpp still names a few of its
// members.  The TraceFEM path driven by oracle/ref_harness.cpp never calls
// them, so every one of those symbols resolves to a function that aborts.
#include <cstdio>
#include <cstdlib>

extern "C" void tf_ref_quaqua_unavailable() {
    std::fputs("ref_harness: QuaQuaMapperCL is not built into the oracle harness\n", stderr);
    std::abort();
}

#define TF_REF_ALIAS(sym) __asm__(".globl " #sym "\n.set " #sym ", tf_ref_quaqua_unavailable\n");
TF_REF_ALIAS(_ZN5DROPS14QuaQuaMapperCLC1ERKS0_)
TF_REF_ALIAS(_ZN5DROPS14QuaQuaMapperCLD1Ev)
TF_REF_ALIAS(_ZN5DROPS7abs_detERKNS_7TetraCLERKNS_9SVectorCLILj4EEERKNS_14QuaQuaMapperCLERKNS_8SPatchCLILj3EEE)
TF_REF_ALIAS(_ZNK5DROPS14QuaQuaMapperCL10base_pointEv)
TF_REF_ALIAS(_ZNK5DROPS14QuaQuaMapperCL13local_ls_gradERKNS_7TetraCLERKNS_9SVectorCLILj4EEE)
TF_REF_ALIAS(_ZNK5DROPS14QuaQuaMapperCL8jacobianEv)
TF_REF_ALIAS(_ZNK5DROPS14QuaQuaMapperCL9set_pointEPKNS_7TetraCLERKNS_9SVectorCLILj4EEE)
