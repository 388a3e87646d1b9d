// Compile-and-link check of the C++ Force-class layer (include/mbpol_gb300.hpp):
// the two-water system of TestReferenceMBPolTwoBodyForce.cpp:99-127.  Run on a
// GPU it prints the two-body energy in kcal/mol (expected 6.14207815).
#include <cstdio>
#include "mbpol_gb300.hpp"

using namespace MBPolPlugin;

int main() {
    System system;
    for (int i = 0; i < 6; ++i) system.addParticle(i % 3 ? 1.008 : 15.999);
    auto* f = new MBPolTwoBodyForce();
    f->setCutoff(10.0);
    f->setNonbondedMethod(MBPolTwoBodyForce::CutoffNonPeriodic);
    f->addParticle({0, 1, 2});
    f->addParticle({3, 4, 5});
    system.addForce(f);
    std::vector<Vec3> pos = {{-1.516074336e-01, -2.023167650e-02, 1.454672917e-01},
                             {-6.218989773e-02, -6.009430735e-02, 1.572437625e-01},
                             {-2.017613812e-01, -4.190350349e-02, 2.239642849e-01},
                             {-1.763651687e-01, -3.816594649e-02, -1.300353949e-01},
                             {-1.903851736e-01, -4.935677617e-02, -3.457810126e-02},
                             {-2.527904158e-01, -7.613550077e-02, -1.733803676e-01}};
    try {
        Context ctx(system);
        ctx.setPositions(pos);
        State st = ctx.getState();
        std::printf("%.8f\n", st.potentialEnergy / 4.184);
    } catch (const MBPolException& e) {
        std::printf("error %d: %s\n", e.status, e.what());
        return e.status == MBPOL_ERR_NO_DEVICE ? 0 : 1;
    }
    return 0;
}
