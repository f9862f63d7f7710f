// Runge-Kutta tableaux of the two steppers on the hot path.
//
// DOP853: Hairer & Wanner's 8(5,3) pair, the values of the reference's
// include/coeff.h:6-176 written as shortest round-trip doubles (identical bits).
// RK45: the 6-stage 4(5) pair of include/coeff.h:178-218 (nodes 2/9, 1/3, 3/4,
// 1, 5/6), each entry the double its rational evaluates to.
#pragma once

namespace st {
namespace dop {
constexpr double C2 = 0.05260015195876773;
constexpr double C3 = 0.0789002279381516;
constexpr double C4 = 0.1183503419072274;
constexpr double C5 = 0.2816496580927726;
constexpr double C6 = 0.3333333333333333;
constexpr double C7 = 0.25;
constexpr double C8 = 0.3076923076923077;
constexpr double C9 = 0.6512820512820513;
constexpr double C10 = 0.6;
constexpr double C11 = 0.8571428571428571;
constexpr double A21 = 0.05260015195876773;
constexpr double A31 = 0.0197250569845379;
constexpr double A32 = 0.0591751709536137;
constexpr double A41 = 0.02958758547680685;
constexpr double A43 = 0.08876275643042054;
constexpr double A51 = 0.2413651341592667;
constexpr double A53 = -0.8845494793282861;
constexpr double A54 = 0.924834003261792;
constexpr double A61 = 0.037037037037037035;
constexpr double A64 = 0.17082860872947386;
constexpr double A65 = 0.12546768756682242;
constexpr double A71 = 0.037109375;
constexpr double A74 = 0.17025221101954405;
constexpr double A75 = 0.06021653898045596;
constexpr double A76 = -0.017578125;
constexpr double A81 = 0.03709200011850479;
constexpr double A84 = 0.17038392571223998;
constexpr double A85 = 0.10726203044637328;
constexpr double A86 = -0.015319437748624402;
constexpr double A87 = 0.008273789163814023;
constexpr double A91 = 0.6241109587160757;
constexpr double A94 = -3.3608926294469414;
constexpr double A95 = -0.868219346841726;
constexpr double A96 = 27.59209969944671;
constexpr double A97 = 20.154067550477894;
constexpr double A98 = -43.48988418106996;
constexpr double A101 = 0.47766253643826434;
constexpr double A104 = -2.4881146199716677;
constexpr double A105 = -0.590290826836843;
constexpr double A106 = 21.230051448181193;
constexpr double A107 = 15.279233632882423;
constexpr double A108 = -33.28821096898486;
constexpr double A109 = -0.020331201708508627;
constexpr double A111 = -0.9371424300859873;
constexpr double A114 = 5.186372428844064;
constexpr double A115 = 1.0914373489967295;
constexpr double A116 = -8.149787010746927;
constexpr double A117 = -18.52006565999696;
constexpr double A118 = 22.739487099350505;
constexpr double A119 = 2.4936055526796523;
constexpr double A1110 = -3.0467644718982196;
constexpr double A121 = 2.273310147516538;
constexpr double A124 = -10.53449546673725;
constexpr double A125 = -2.0008720582248625;
constexpr double A126 = -17.9589318631188;
constexpr double A127 = 27.94888452941996;
constexpr double A128 = -2.8589982771350235;
constexpr double A129 = -8.87285693353063;
constexpr double A1210 = 12.360567175794303;
constexpr double A1211 = 0.6433927460157636;
constexpr double B1 = 0.054293734116568765;
constexpr double B6 = 4.450312892752409;
constexpr double B7 = 1.8915178993145003;
constexpr double B8 = -5.801203960010585;
constexpr double B9 = 0.3111643669578199;
constexpr double B10 = -0.1521609496625161;
constexpr double B11 = 0.20136540080403034;
constexpr double B12 = 0.04471061572777259;
constexpr double BHH1 = 0.2440944881889764;
constexpr double BHH2 = 0.7338466882816118;
constexpr double BHH3 = 0.022058823529411766;
constexpr double ER1 = 0.01312004499419488;
constexpr double ER6 = -1.2251564463762044;
constexpr double ER7 = -0.4957589496572502;
constexpr double ER8 = 1.6643771824549864;
constexpr double ER9 = -0.35032884874997366;
constexpr double ER10 = 0.3341791187130175;
constexpr double ER11 = 0.08192320648511571;
constexpr double ER12 = -0.022355307863886294;
}  // namespace dop
namespace rk45 {
constexpr double A2 = 0.2222222222222222;
constexpr double A3 = 0.3333333333333333;
constexpr double A4 = 0.75;
constexpr double A5 = 1.0;
constexpr double A6 = 0.8333333333333334;
constexpr double B21 = 0.2222222222222222;
constexpr double B31 = 0.08333333333333333;
constexpr double B32 = 0.25;
constexpr double B41 = 0.5390625;
constexpr double B42 = -1.8984375;
constexpr double B43 = 2.109375;
constexpr double B51 = -1.4166666666666667;
constexpr double B52 = 6.75;
constexpr double B53 = -5.4;
constexpr double B54 = 1.0666666666666667;
constexpr double B61 = 0.15046296296296297;
constexpr double B62 = -0.3125;
constexpr double B63 = 0.8125;
constexpr double B64 = 0.14814814814814814;
constexpr double B65 = 0.034722222222222224;
constexpr double CH1 = 0.10444444444444445;
constexpr double CH2 = 0.0;
constexpr double CH3 = 0.48;
constexpr double CH4 = 0.14222222222222222;
constexpr double CH5 = 0.03333333333333333;
constexpr double CH6 = 0.24;
constexpr double CT1 = 0.006666666666666667;
constexpr double CT2 = 0.0;
constexpr double CT3 = -0.03;
constexpr double CT4 = 0.21333333333333335;
constexpr double CT5 = 0.05;
constexpr double CT6 = -0.24;
// step-size controller exponents beta1/k and beta2/k (src/integrator.cpp:262-265)
constexpr double E1 = 0.7 / 7.0;
constexpr double E2 = -0.4 / 7.0;
}  // namespace rk45
}  // namespace st
