3
Al V upsilions from Saraph H.E. Tully J.A. (A&A Suppl.,107,29,1994)
 Si VI  Collision strengths from K. Butler (in preparation).
        Aij from NSRDS-NBS 22, Vol. II  (entered by MJB 12-Feb-1990)
2 10 0
 2P3
 2P1
1000
1778
3162
5623
10000
17783
31623
56234
100000
177828
 0
 1 2 .381  
 0 0 .386
 0 0 .403
 0 0 .450
 0 0 .506
 0 0 .524
 0 0 .502
 0 0 .474
 0 0 .464
 0 0 .459
0 0 0
 1 2 .731
 1 4 0
 2 2 3443.7
