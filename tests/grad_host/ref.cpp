// Reference contracted ERIs for the host check of the gradient bodies: a
// direct McMurchie-Davidson evaluation (runtime loops, recursive R, Boys
// function by its convergent series) independent of the generated code.
#include "common.h"
using namespace hfgpu;
// plain McMurchie-Davidson reference: contracted (ab|cd) for all components
static double boysF(int m, double T) {
    // series F_m(T) = e^-T sum (2T)^i / ((2m+1)(2m+3)...(2m+2i+1))
    if (T > 30) { double f = 0.5*std::sqrt(M_PI/T); for (int k=0;k<m;k++) f = f*(2*k+1)/(2*T); return f; }
    double term = 1.0/(2*m+1), s = term;
    for (int i=1;i<200;i++){ term *= 2*T/(2*m+2*i+1); s += term; if (term < 1e-18*s) break; }
    return std::exp(-T)*s;
}
static void e1d(double E[6][6][12], int imax, int jmax, double xpa, double xpb, double p) {
    for (int i=0;i<6;i++) for(int j=0;j<6;j++) for(int t=0;t<12;t++) E[i][j][t]=0;
    E[0][0][0] = 1;
    for (int i=0;i<=imax;i++) for (int j=0;j<=jmax;j++) {
        if (i==0 && j==0) continue;
        for (int t=0;t<=i+j;t++) {
            double v;
            if (i>0) { v = xpa*E[i-1][j][t] + (t>0? E[i-1][j][t-1]/(2*p):0) + (t+1<=i-1+j? (t+1)*E[i-1][j][t+1]:0); }
            else { v = xpb*E[i][j-1][t] + (t>0? E[i][j-1][t-1]/(2*p):0) + (t+1<=i+j-1? (t+1)*E[i][j-1][t+1]:0); }
            E[i][j][t] = v;
        }
    }
}
static double Rn(int n, int t, int u, int v, double al, double X, double Y, double Z, const double* F) {
    if (t<0||u<0||v<0) return 0;
    if (t==0&&u==0&&v==0) return std::pow(-2*al, n)*F[n];
    if (t>0) return (t>1?(t-1)*Rn(n+1,t-2,u,v,al,X,Y,Z,F):0) + X*Rn(n+1,t-1,u,v,al,X,Y,Z,F);
    if (u>0) return (u>1?(u-1)*Rn(n+1,t,u-2,v,al,X,Y,Z,F):0) + Y*Rn(n+1,t,u-1,v,al,X,Y,Z,F);
    return (v>1?(v-1)*Rn(n+1,t,u,v-2,al,X,Y,Z,F):0) + Z*Rn(n+1,t,u,v-1,al,X,Y,Z,F);
}
// full block [a][b][c][d]
std::vector<double> ref_block(const Shell& A, const Shell& B, const Shell& C, const Shell& D) {
    int NA=ncart(A.L),NB=ncart(B.L),NC=ncart(C.L),ND=ncart(D.L);
    std::vector<double> out((size_t)NA*NB*NC*ND, 0.0);
    static double Eab[3][6][6][12], Ecd[3][6][6][12];
    int L = A.L+B.L+C.L+D.L;
    for (size_t ia=0;ia<A.a.size();ia++) for (size_t ib=0;ib<B.a.size();ib++)
    for (size_t ic=0;ic<C.a.size();ic++) for (size_t id=0;id<D.a.size();id++) {
        double a=A.a[ia],b=B.a[ib],c=C.a[ic],d=D.a[id];
        double p=a+b,q=c+d, P[3],Q[3], rab2=0, rcd2=0;
        for (int k=0;k<3;k++){ P[k]=(a*A.c[k]+b*B.c[k])/p; Q[k]=(c*C.c[k]+d*D.c[k])/q; rab2+=(A.c[k]-B.c[k])*(A.c[k]-B.c[k]); rcd2+=(C.c[k]-D.c[k])*(C.c[k]-D.c[k]); }
        for (int k=0;k<3;k++){ e1d(Eab[k],A.L,B.L,P[k]-A.c[k],P[k]-B.c[k],p); e1d(Ecd[k],C.L,D.L,Q[k]-C.c[k],Q[k]-D.c[k],q); }
        double al=p*q/(p+q); double X=P[0]-Q[0],Y=P[1]-Q[1],Z=P[2]-Q[2];
        double T=al*(X*X+Y*Y+Z*Z); double F[16]; for(int m=0;m<=L;m++) F[m]=boysF(m,T);
        double pre = 2*std::pow(M_PI,2.5)/(p*q*std::sqrt(p+q))*std::exp(-a*b/p*rab2)*std::exp(-c*d/q*rcd2);
        for (int ca=0;ca<NA;ca++) for(int cb=0;cb<NB;cb++) for(int cc=0;cc<NC;cc++) for(int cd=0;cd<ND;cd++){
            Cart x1=cart(A.L,ca),x2=cart(B.L,cb),x3=cart(C.L,cc),x4=cart(D.L,cd);
            double s=0;
            for(int t=0;t<=x1.l+x2.l;t++)for(int u=0;u<=x1.m+x2.m;u++)for(int v=0;v<=x1.n+x2.n;v++){
                double e1=Eab[0][x1.l][x2.l][t]*Eab[1][x1.m][x2.m][u]*Eab[2][x1.n][x2.n][v];
                for(int t2=0;t2<=x3.l+x4.l;t2++)for(int u2=0;u2<=x3.m+x4.m;u2++)for(int v2=0;v2<=x3.n+x4.n;v2++){
                    double e2=Ecd[0][x3.l][x4.l][t2]*Ecd[1][x3.m][x4.m][u2]*Ecd[2][x3.n][x4.n][v2];
                    double sg=((t2+u2+v2)&1)?-1:1;
                    s+=e1*e2*sg*Rn(0,t+t2,u+u2,v+v2,al,X,Y,Z,F);
                }
            }
            double co = A.co[ca*A.a.size()+ia]*B.co[cb*B.a.size()+ib]*C.co[cc*C.a.size()+ic]*D.co[cd*D.a.size()+id];
            out[((size_t)(ca*NB+cb)*NC+cc)*ND+cd] += pre*co*s;
        }
    }
    return out;
}
