// Runge-Kutta tableaux of the two steppers on the hot path.
//
// DOP853: Hairer & Wanner's 8(5,3) pair, the values of the reference's
// include/coeff.h:6-176 written as shortest round-trip doubles (identical bits).
// RK45: the 6-stage 4(5) pair of include/coeff.h:178-218 (nodes 2/9, 1/3, 3/4,
// 1, 5/6), each entry the double its rational evaluates to.
// RKF45: Fehlberg's 4(5) pair of include/coeff.h:220-255; CFET8 / CFET6: the
// commutator-free exponential integrators of orders 8 and 6 on the 5-point
// Gauss-Legendre nodes (include/coeff.h:257-320), used by the Magnus stepper.
// Both written as shortest round-trip doubles of the reference's values.
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
// fourth-order weights (the quaternion form's error estimate; C2 = 0)
constexpr double C1 = 0.1111111111111111;
constexpr double C3 = 0.45;
constexpr double C4 = 0.35555555555555557;
constexpr double C5 = 0.08333333333333333;
// step-size controller exponents beta1/k and beta2/k (src/integrator.cpp:262-265)
constexpr double E1 = 0.7 / 7.0;
constexpr double E2 = -0.4 / 7.0;
}  // namespace rk45

namespace rkf45 {
constexpr double A2 = 0.25;
constexpr double A3 = 0.375;
constexpr double A4 = 0.9230769230769231;
constexpr double A5 = 1.0;
constexpr double A6 = 0.5;
constexpr double B21 = 0.25;
constexpr double B31 = 0.09375;
constexpr double B32 = 0.28125;
constexpr double B41 = 0.8793809740555303;
constexpr double B42 = -3.277196176604461;
constexpr double B43 = 3.3208921256258535;
constexpr double B51 = 2.0324074074074074;
constexpr double B52 = -8.0;
constexpr double B53 = 7.173489278752436;
constexpr double B54 = -0.20589668615984405;
constexpr double B61 = -0.2962962962962963;
constexpr double B62 = 2.0;
constexpr double B63 = -1.3816764132553607;
constexpr double B64 = 0.4529727095516569;
constexpr double B65 = -0.275;
// fifth-order weights (C2 = 0) and fourth-order weights (CR2 = CR6 = 0)
constexpr double C1 = 0.11851851851851852;
constexpr double C3 = 0.5189863547758284;
constexpr double C4 = 0.5061314903420167;
constexpr double C5 = -0.18;
constexpr double C6 = 0.03636363636363636;
constexpr double CR1 = 0.11574074074074074;
constexpr double CR3 = 0.5489278752436647;
constexpr double CR4 = 0.5353313840155945;
constexpr double CR5 = -0.2;
}  // namespace rkf45

namespace cfet {
// Gauss-Legendre nodes on [0, 1]
constexpr double X1 = 0.046910077030668074;
constexpr double X2 = 0.2307653449471585;
constexpr double X3 = 0.5;
constexpr double X4 = 0.7692346550528415;
constexpr double X5 = 0.9530899229693319;
// CFET8: exponent j (1-6) weights the five node fields by row j; exponents
// 7-11 take rows 5..1 with the node order reversed
constexpr double G11 = -0.005984812750244602;
constexpr double G12 = 0.020217897716672675;
constexpr double G13 = -0.03646660716686794;
constexpr double G14 = 0.04245408899634467;
constexpr double G15 = 0.14949496424802844;
constexpr double G21 = 0.02512881778391826;
constexpr double G22 = -0.08955337580937157;
constexpr double G23 = 0.19032828600393248;
constexpr double G24 = 0.28920194841768715;
constexpr double G25 = -0.03568486888016069;
constexpr double G31 = -0.04972613261435144;
constexpr double G32 = 0.6572496090804754;
constexpr double G33 = 0.11725149008224456;
constexpr double G34 = -0.43611911073577403;
constexpr double G35 = 0.18080345083145516;
constexpr double G41 = 0.0464837870954061;
constexpr double G42 = -0.6265183532355708;
constexpr double G43 = -0.11144873822286155;
constexpr double G44 = 0.4154988625423615;
constexpr double G45 = -0.17224148557040517;
constexpr double G51 = 0.015567390500242426;
constexpr double G52 = -0.0677120111619075;
constexpr double G53 = -0.15241336773272682;
constexpr double G54 = -0.08803798509100481;
constexpr double G55 = -0.0013284996209207986;
constexpr double G61 = -0.034049168494873015;
constexpr double G62 = 0.12263276452977083;
constexpr double G63 = 0.2699423185170027;
constexpr double G64 = 0.12263276452977094;
constexpr double G65 = -0.03404916849487304;
// CFET6: exponents 1-3 by row, 4-5 take rows 2, 1 reversed
constexpr double H11 = -0.007431519425246311;
constexpr double H12 = 0.022452824849980513;
constexpr double H13 = -0.03620393417193995;
constexpr double H14 = 0.0409779901800809;
constexpr double H15 = 0.1516046385671249;
constexpr double H21 = 0.03095749686312404;
constexpr double H22 = -0.10116885619385878;
constexpr double H23 = 0.1997455955716367;
constexpr double H24 = 0.3010242365525433;
constexpr double H25 = -0.055594729593982636;
constexpr double H31 = -0.001072443882925378;
constexpr double H32 = -0.023971860139062367;
constexpr double H33 = -0.04263887835494916;
constexpr double H34 = -0.023971860139062388;
constexpr double H35 = -0.0010724438829253797;
}  // namespace cfet
}  // namespace st
