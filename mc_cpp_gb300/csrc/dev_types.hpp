// Plain parameter blocks passed by value to the kernels (usable from host C++ and CUDA).
#pragma once

namespace mcg {

struct PbcDev {
    int type;           // 0 none, 1 cubic, 2 orthorhombic
    double L[3], rL[3];
};

struct CutDev {
    int mode;           // 0 full, 1 switch
    double c2, n2, sw2; // cutoff^2, cuton^2, 1/(c2-n2)^3
    float c2f, n2f, sw2f;
};

}  // namespace mcg
