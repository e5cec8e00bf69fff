/* cntc_host.c -- a C host of the library: the steady-rolling case of CONTACT's module 3
 * (Hertzian 6 x 4 mm contact, steel on steel, Fn 100 kN, creepage 0.001, mu 0.3) through the
 * plain C-ABI of include/contact_addon.h, the way the reference's C example drives it.
 *
 *   cntc_host            set-up and getters only (no device needed)
 *   cntc_host solve N    also cntc_calculate on an N x N grid, GDsteady, eps 1e-10; prints
 *                        ierror, forces, penetration, maximum pressure and element counts
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "contact_addon.h"

int main(int argc, char **argv) {
    int solve = argc > 1 && strcmp(argv[1], "solve") == 0;
    int m = (argc > 2) ? atoi(argv[2]) : 21;
    int ire = 1, icp = 1, imodul = 3, ifcver = 0, ierror = 0, ioutput = 0, len = 1;
    cntc_initializefirst_new(&ifcver, &ierror, &ioutput, " ", " ", " ", &len, &len, &len);
    cntc_initialize(&ire, &imodul, &ifcver, &ierror, " ", &len);
    if (ierror != 0) { printf("initialize ierror %d\n", ierror); return 1; }

    int flags[3] = {1972 /* CNTC_ic_tang */, 1971 /* CNTC_ic_bound */, 1983 /* CNTC_ic_iestim */};
    int fvals[3] = {3, 0, 0};
    int nflag = 3;
    cntc_setflags(&ire, &icp, &nflag, flags, fvals);
    int mdigit = 0, nmat = 4;
    double mat[4] = {0.28, 0.28, 82031.25, 82031.25};
    cntc_setmaterialparameters(&ire, &icp, &mdigit, &nmat, mat);
    int lmeth = 0, nfric = 2;
    double fric[2] = {0.3, 0.3};
    cntc_setfrictionmethod(&ire, &icp, &lmeth, &nfric, fric);
    double veloc = 10000.0;
    cntc_setreferencevelocity(&ire, &icp, &veloc);
    int gdigit = 5, nints = 5, nreals = 8;
    int iparam[5] = {999, 100, 30, 1, 1};
    double rparam[8] = {1e-10, 0.9, 0.1, 1.0, 1.0, 1.0, 1.0, 0.9};
    cntc_setsolverflags(&ire, &icp, &gdigit, &nints, iparam, &nreals, rparam);
    int ipotcn = -3, nhz = 5;
    double hz[5] = {(double)m, (double)m, 6.0, 4.0, 1.1};
    cntc_sethertzcontact(&ire, &icp, &ipotcn, &nhz, hz);
    double fn = 1e5, cksi = 0.001, ceta = 0.0, cphi = 0.0;
    cntc_setnormalforce(&ire, &icp, &fn);
    cntc_setcreepages(&ire, &icp, &cksi, &ceta, &cphi);

    double vx = 0, vy = 0, phi = 0;
    cntc_getcreepages(&ire, &icp, &vx, &vy, &phi);
    int qflags[2] = {1972, 1973 /* CNTC_ic_norm */}, qvals[2] = {0, 0}, nq = 2;
    cntc_getflags(&ire, &icp, &nq, qflags, qvals);
    printf("setup tang %d norm %d creep %.6g %.6g %.6g\n", qvals[0], qvals[1], vx, vy, phi);

    if (solve) {
        cntc_calculate(&ire, &icp, &ierror);
        double ffn = 0, fx = 0, fy = 0, mz = 0, pen = 0, pmax = 0;
        cntc_getcontactforces(&ire, &icp, &ffn, &fx, &fy, &mz);
        cntc_getpenetration(&ire, &icp, &pen);
        cntc_getmaximumpressure(&ire, &icp, &pmax);
        int mx = 0, my = 0;
        cntc_getnumelements(&ire, &icp, &mx, &my);
        int n = mx * my;
        int *eldiv = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
        cntc_getelementdivision(&ire, &icp, &n, eldiv);
        int nadh = 0, nslip = 0;
        for (int i = 0; i < n; i++) { nadh += eldiv[i] == 1; nslip += eldiv[i] == 2; }
        free(eldiv);
        printf("solve ierror %d fn %.17g fx %.17g fy %.17g mz %.17g pen %.17g pmax %.17g nadh %d nslip %d\n",
               ierror, ffn, fx, fy, mz, pen, pmax, nadh, nslip);
    }
    cntc_finalize(&ire);
    cntc_finalizelast();
    return 0;
}
