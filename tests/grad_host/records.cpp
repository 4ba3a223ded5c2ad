// Pair records for the host check of the gradient bodies, laid out as the
// device builds them: the bra side as grad_pair_kernel (grad.cu) writes them,
// the ket side as pair_data_kernel (eri.cu) writes the energy records.
#include "common.h"
using namespace hfgpu;
static void e1d(double E[6][6][12], int imax, int jmax, double xpa, double xpb, double p) {
    for (int i=0;i<6;i++) for(int j=0;j<6;j++) for(int t=0;t<12;t++) E[i][j][t]=0;
    E[0][0][0] = 1;
    for (int i=0;i<=imax;i++) for (int j=0;j<=jmax;j++) {
        if (i==0 && j==0) continue;
        for (int t=0;t<=i+j;t++) {
            double v;
            if (i>0) v = xpa*E[i-1][j][t] + (t>0? E[i-1][j][t-1]/(2*p):0) + (t+1<=i-1+j? (t+1)*E[i-1][j][t+1]:0);
            else v = xpb*E[i][j-1][t] + (t>0? E[i][j-1][t-1]/(2*p):0) + (t+1<=i+j-1? (t+1)*E[i][j-1][t+1]:0);
            E[i][j][t] = v;
        }
    }
}
void boys_row(int M, double T, double* F) {
    for (int m = 0; m <= M; ++m) {
        if (T > 30) { double f = 0.5*std::sqrt(M_PI/T); for (int k=0;k<m;k++) f = f*(2*k+1)/(2*T); F[m] = f; continue; }
        double term = 1.0/(2*m+1), s = term;
        for (int i=1;i<200;i++){ term *= 2*T/(2*m+2*i+1); s += term; if (term < 1e-18*s) break; }
        F[m] = std::exp(-T)*s;
    }
}
void make_records(const Shell& A, const Shell& B, const Shell& C, const Shell& D, std::vector<double>& gb,
                  std::vector<double>& ek, int& nbp, int& nkp) {
    int la = A.L, lb = B.L, lc = C.L, ld = D.L;
    static double E[3][6][6][12];
    nbp = A.a.size() * B.a.size();
    nkp = C.a.size() * D.a.size();
    int SG = grad_stride(la, lb), SK = pair_stride(lc, ld);
    gb.assign((size_t)nbp * SG, 0.0);
    ek.assign((size_t)nkp * SK, 0.0);
    int ts = grad_table(la, lb), tw = la + lb + 2;
    for (size_t ia = 0; ia < A.a.size(); ++ia) for (size_t ib = 0; ib < B.a.size(); ++ib) {
        double a = A.a[ia], b = B.a[ib], p = a + b, P[3], rab2 = 0;
        for (int k = 0; k < 3; ++k) { P[k] = (a*A.c[k] + b*B.c[k]) / p; rab2 += (A.c[k]-B.c[k])*(A.c[k]-B.c[k]); }
        double kab = std::exp(-a*b/p*rab2) / p;
        double* r = gb.data() + (ia * B.a.size() + ib) * SG;
        r[0]=a; r[1]=b; r[2]=p; r[3]=P[0]; r[4]=P[1]; r[5]=P[2]; r[6]=kab;
        for (int c = 0; c < ncart(la); ++c) r[8+c] = A.co[c*A.a.size()+ia]*kab;
        for (int c = 0; c < ncart(lb); ++c) r[14+c] = B.co[c*B.a.size()+ib];
        for (int d = 0; d < 3; ++d) {
            e1d(E[d], la+1, lb, P[d]-A.c[d], P[d]-B.c[d], p);
            for (int i=0;i<=la;i++) for(int j=0;j<=lb;j++) for (int t=0;t<tw;t++) {
                int o = (i*(lb+1)+j)*tw + t;
                r[GR_HDR + d*ts + o] = t <= i+j ? E[d][i][j][t] : 0.0;
                r[GR_HDR + (3+d)*ts + o] = 2*a*E[d][i+1][j][t] - (i>0 ? i*E[d][i-1][j][t] : 0.0);
            }
        }
    }
    for (size_t ic = 0; ic < C.a.size(); ++ic) for (size_t id = 0; id < D.a.size(); ++id) {
        double c = C.a[ic], d = D.a[id], q = c + d, Q[3], rcd2 = 0;
        for (int k = 0; k < 3; ++k) { Q[k] = (c*C.c[k] + d*D.c[k]) / q; rcd2 += (C.c[k]-D.c[k])*(C.c[k]-D.c[k]); }
        double kcd = std::exp(-c*d/q*rcd2) / q;
        for (int k = 0; k < 3; ++k) e1d(E[k], lc, ld, Q[k]-C.c[k], Q[k]-D.c[k], q);
        double* r = ek.data() + (ic * D.a.size() + id) * SK;
        r[0]=q; r[1]=Q[0]; r[2]=Q[1]; r[3]=Q[2];
        for (int cc = 0; cc < ncart(lc); ++cc) for (int cd = 0; cd < ncart(ld); ++cd) {
            Cart x = cart(lc, cc), y = cart(ld, cd);
            double s = C.co[cc*C.a.size()+ic]*D.co[cd*D.a.size()+id]*kcd;
            double* e = r + PAIR_HDR + eoff(lc, ld, cc, cd);
            int w = 0;
            for (int t=0;t<=x.l+y.l;t++) for(int u=0;u<=x.m+y.m;u++) for(int v=0;v<=x.n+y.n;v++)
                e[w++] = s*E[0][x.l][y.l][t]*E[1][x.m][y.m][u]*E[2][x.n][y.n][v];
        }
    }
}
