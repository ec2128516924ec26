NAME          BASIC
ROWS
 N  COST
 L  LIM1
 G  LIM2
 E  MYEQN
COLUMNS
    X1        COST         1.0   LIM1         1.0
    X1        LIM2         1.0
    X2        COST         2.0   LIM1         1.0
    X2        MYEQN       -1.0
    X3        COST        -1.0   MYEQN        1.0
RHS
    RHS       COST        -3.5
    RHS       LIM1         4.0   LIM2         1.0
    RHS       MYEQN        7.0
RANGES
    RNG       LIM1         2.5   MYEQN       -3
BOUNDS
 UP BND       X1           4.0
 MI BND       X2
 UP BND       X2           1.0
 FX BND       X3           2.5
ENDATA
