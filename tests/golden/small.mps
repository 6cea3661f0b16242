NAME          SMALL
ROWS
 N  COST
 E  EQ1
 E  EQ2
 E  EQ3
 E  EQ4
 E  EQ5
 E  EQ6
 E  EQ7
 E  EQ8
 E  EQ9
 E  EQ10
 E  EQ11
 E  EQ12
 E  EQ13
 E  EQ14
 E  EQ15
 E  EQ16
 E  EQ17
 E  EQ18
 E  EQ19
 E  EQ20
 E  EQ21
 E  EQ22
 E  EQ23
 E  EQ24
 E  EQ25
 E  EQ26
 E  EQ27
 E  EQ28
 E  EQ29
 E  EQ30
 E  EQ31
 E  EQ32
 E  EQ33
 E  EQ34
 E  EQ35
 E  EQ36
 E  EQ37
 E  EQ38
 E  EQ39
 E  EQ40
 E  EQ41
 E  EQ42
 E  EQ43
 E  EQ44
 E  EQ45
 E  EQ46
 E  EQ47
 E  EQ48
 E  EQ49
 E  EQ50
 E  EQ51
 E  EQ52
 E  EQ53
 E  EQ54
 E  EQ55
 E  EQ56
 E  EQ57
 E  EQ58
 E  EQ59
 E  EQ60
 E  EQ61
 E  EQ62
 E  EQ63
 E  EQ64
 E  EQ65
 E  EQ66
 E  EQ67
 E  EQ68
 E  EQ69
 E  EQ70
 E  EQ71
 E  EQ72
COLUMNS
    X1        EQ3       -2          
    X1        EQ36      -1          
    X1        EQ53      2           
    X1        EQ68      -1          
    X2        EQ19      -2          
    X2        EQ30      -2          
    X2        EQ58      2           
    X3        EQ24      -1          
    X3        EQ33      2           
    X3        EQ38      -2          
    X3        EQ57      -1          
    X3        EQ58      -1          
    X4        EQ2       1           
    X4        EQ5       2           
    X4        EQ14      -2          
    X4        EQ19      1           
    X4        EQ35      -1          
    X4        EQ54      1           
    X5        EQ12      -1          
    X5        EQ19      2           
    X5        EQ23      -1          
    X5        EQ31      1           
    X5        EQ50      2           
    X5        EQ69      2           
    X6        EQ3       -1          
    X6        EQ38      1           
    X6        EQ51      2           
    X6        EQ63      2           
    X7        EQ19      1           
    X7        EQ42      1           
    X7        EQ58      1           
    X8        EQ4       1           
    X8        EQ11      2           
    X8        EQ53      2           
    X8        EQ68      2           
    X9        EQ40      -2          
    X9        EQ58      -1          
    X10       EQ16      2           
    X10       EQ62      2           
    X11       EQ1       2           
    X11       EQ20      2           
    X11       EQ21      -1          
    X11       EQ33      -1          
    X11       EQ43      -2          
    X11       EQ66      1           
    X12       EQ56      2           
    X12       EQ58      2           
    X12       EQ65      -1          
    X12       EQ69      1           
    X12       EQ71      1           
    X13       EQ2       -1          
    X13       EQ32      -2          
    X13       EQ34      1           
    X13       EQ47      2           
    X13       EQ66      2           
    X13       EQ69      -2          
    X14       EQ5       -2          
    X14       EQ22      1           
    X14       EQ34      1           
    X14       EQ55      -2          
    X14       EQ56      1           
    X14       EQ59      -1          
    X15       EQ1       -1          
    X15       EQ19      1           
    X15       EQ40      2           
    X15       EQ45      -1          
    X16       EQ37      -2          
    X16       EQ52      -1          
    X17       EQ6       2           
    X17       EQ20      2           
    X17       EQ22      -2          
    X17       EQ44      -2          
    X17       EQ58      -2          
    X17       EQ59      -1          
    X18       EQ6       -2          
    X18       EQ19      1           
    X18       EQ64      2           
    X19       EQ10      -1          
    X19       EQ28      -1          
    X20       EQ16      -1          
    X20       EQ32      -1          
    X20       EQ33      -1          
    X20       EQ39      1           
    X20       EQ42      -1          
    X21       EQ4       -1          
    X21       EQ8       -1          
    X22       EQ23      2           
    X22       EQ52      1           
    X23       EQ64      -2          
    X23       EQ69      2           
    X24       EQ25      1           
    X24       EQ42      -2          
    X24       EQ50      -2          
    X24       EQ52      -1          
    X24       EQ67      1           
    X25       EQ10      2           
    X25       EQ19      2           
    X25       EQ66      -1          
    X26       EQ7       1           
    X26       EQ11      2           
    X26       EQ37      2           
    X26       EQ52      -2          
    X26       EQ54      2           
    X26       EQ64      1           
    X27       EQ13      2           
    X27       EQ17      2           
    X27       EQ28      -2          
    X27       EQ64      1           
    X27       EQ67      2           
    X28       EQ11      -2          
    X28       EQ22      -2          
    X28       EQ36      2           
    X28       EQ38      1           
    X28       EQ41      2           
    X29       EQ25      -2          
    X29       EQ28      -1          
    X29       EQ45      1           
    X29       EQ46      2           
    X29       EQ59      2           
    X29       EQ72      -1          
    X30       EQ32      -1          
    X30       EQ52      -2          
    X30       EQ62      2           
    X30       EQ72      -1          
    X31       EQ17      -2          
    X31       EQ19      2           
    X31       EQ28      1           
    X31       EQ69      1           
    X32       EQ26      -1          
    X32       EQ29      -1          
    X32       EQ55      2           
    X32       EQ67      -1          
    X33       EQ9       1           
    X33       EQ11      1           
    X33       EQ16      -1          
    X33       EQ26      2           
    X33       EQ41      -2          
    X34       EQ7       -2          
    X34       EQ18      2           
    X34       EQ21      2           
    X34       EQ25      -1          
    X34       EQ42      1           
    X35       EQ5       2           
    X35       EQ38      -2          
    X35       EQ54      -1          
    X35       EQ61      1           
    X36       EQ1       1           
    X36       EQ12      1           
    X36       EQ40      1           
    X36       EQ42      -2          
    X37       EQ10      1           
    X37       EQ20      -2          
    X37       EQ31      1           
    X37       EQ49      1           
    X37       EQ69      -1          
    X38       EQ20      1           
    X38       EQ68      1           
    X38       EQ69      2           
    X38       EQ72      -1          
    X39       EQ2       -1          
    X39       EQ7       1           
    X39       EQ9       -1          
    X39       EQ26      2           
    X39       EQ46      -1          
    X39       EQ59      1           
    X40       EQ54      1           
    X40       EQ58      -2          
    X41       EQ3       -1          
    X41       EQ31      -2          
    X41       EQ32      -2          
    X41       EQ52      -1          
    X41       EQ70      -2          
    X42       EQ16      -2          
    X42       EQ28      -1          
    X43       EQ2       1           
    X43       EQ10      2           
    X43       EQ22      2           
    X43       EQ42      2           
    X43       EQ46      2           
    X43       EQ60      -1          
    X44       EQ9       2           
    X44       EQ10      2           
    X44       EQ25      -2          
    X44       EQ27      1           
    X44       EQ33      2           
    X44       EQ34      -2          
    X45       EQ9       2           
    X45       EQ67      -2          
    X46       EQ3       -1          
    X46       EQ9       2           
    X46       EQ38      -2          
    X46       EQ43      1           
    X46       EQ44      1           
    X47       EQ2       1           
    X47       EQ12      2           
    X47       EQ34      2           
    X47       EQ55      -2          
    X47       EQ60      -1          
    X48       EQ5       2           
    X48       EQ12      -1          
    X48       EQ29      -1          
    X48       EQ46      -1          
    X48       EQ51      2           
    X48       EQ66      1           
    X49       EQ18      1           
    X49       EQ33      -1          
    X49       EQ67      2           
    X49       EQ70      1           
    X50       EQ18      -1          
    X50       EQ29      1           
    X50       EQ37      -2          
    X50       EQ43      1           
    X51       EQ5       2           
    X51       EQ15      -2          
    X52       EQ1       -2          
    X52       EQ8       -2          
    X52       EQ10      -1          
    X52       EQ21      -2          
    X52       EQ46      -2          
    X52       EQ68      -2          
    X53       EQ19      -2          
    X53       EQ24      -1          
    X53       EQ41      -1          
    X53       EQ59      2           
    X54       EQ10      -1          
    X54       EQ53      2           
    X54       EQ61      2           
    X55       EQ12      -2          
    X55       EQ46      2           
    X56       EQ13      -1          
    X56       EQ27      -1          
    X56       EQ36      1           
    X57       EQ15      -2          
    X57       EQ20      -2          
    X57       EQ29      -1          
    X57       EQ54      -1          
    X57       EQ64      1           
    X57       EQ69      -1          
    X58       EQ14      1           
    X58       EQ36      -2          
    X58       EQ43      -2          
    X58       EQ53      2           
    X59       EQ12      -1          
    X59       EQ57      -2          
    X59       EQ67      -1          
    X60       EQ9       1           
    X60       EQ16      2           
    X60       EQ31      -2          
    X60       EQ46      -2          
    X61       EQ5       -2          
    X61       EQ39      -2          
    X61       EQ68      2           
    X62       EQ39      2           
    X62       EQ50      -1          
    X63       EQ43      -1          
    X63       EQ59      -2          
    X63       EQ67      1           
    X64       EQ21      -2          
    X64       EQ28      -2          
    X64       EQ45      -1          
    X64       EQ51      -2          
    X65       EQ27      2           
    X65       EQ40      -1          
    X65       EQ53      -1          
    X65       EQ67      -1          
    X65       EQ71      -1          
    X66       EQ2       -2          
    X66       EQ20      1           
    X66       EQ51      1           
    X66       EQ67      -2          
    X66       EQ70      2           
    X67       EQ14      -1          
    X67       EQ39      1           
    X67       EQ69      2           
    X68       EQ3       -1          
    X68       EQ12      1           
    X68       EQ27      -1          
    X68       EQ40      2           
    X68       EQ43      1           
    X68       EQ46      -2          
    X69       EQ32      1           
    X69       EQ36      1           
    X69       EQ48      -1          
    X70       EQ35      -1          
    X70       EQ36      1           
    X70       EQ37      1           
    X71       EQ11      -2          
    X71       EQ20      1           
    X71       EQ31      -2          
    X71       EQ69      1           
    X71       EQ71      2           
    X72       EQ2       1           
    X72       EQ8       1           
    X72       EQ11      -2          
    X72       EQ14      -1          
    X72       EQ29      1           
    X72       EQ70      -2          
    X73       EQ30      -2          
    X73       EQ45      -2          
    X73       EQ67      -2          
    X73       EQ71      -2          
    X74       EQ11      2           
    X74       EQ21      1           
    X74       EQ23      -2          
    X74       EQ26      2           
    X74       EQ27      -2          
    X74       EQ54      1           
    X75       EQ9       1           
    X75       EQ17      1           
    X75       EQ21      2           
    X75       EQ28      -2          
    X75       EQ64      2           
    X76       EQ41      -1          
    X76       EQ49      2           
    X76       EQ51      1           
    X76       EQ52      2           
    X76       EQ58      1           
    X77       EQ7       -1          
    X77       EQ22      -2          
    X77       EQ28      -1          
    X77       EQ29      -1          
    X77       EQ48      -2          
    X77       EQ62      1           
    X78       EQ22      -2          
    X78       EQ44      1           
    X78       EQ56      -1          
    X79       EQ26      -2          
    X79       EQ30      2           
    X79       EQ36      1           
    X79       EQ42      2           
    X79       EQ47      2           
    X79       EQ63      -2          
    X80       EQ57      2           
    X80       EQ70      -1          
    X81       EQ2       1           
    X81       EQ7       1           
    X81       EQ12      1           
    X81       EQ21      -1          
    X81       EQ23      1           
    X81       EQ54      -2          
    X82       EQ24      -1          
    X82       EQ26      -1          
    X82       EQ62      2           
    X83       EQ21      -1          
    X83       EQ38      -1          
    X83       EQ59      -1          
    X83       EQ64      -2          
    X83       EQ68      2           
    X84       EQ10      -2          
    X84       EQ27      1           
    X85       EQ10      -2          
    X85       EQ31      -1          
    X85       EQ44      2           
    X86       EQ2       -1          
    X86       EQ4       1           
    X86       EQ23      2           
    X86       EQ44      -1          
    X86       EQ71      2           
    X87       EQ4       2           
    X87       EQ25      2           
    X87       EQ55      -2          
    X87       EQ69      1           
    X88       EQ48      -1          
    X88       EQ52      2           
    X88       EQ58      -2          
    X89       EQ7       2           
    X89       EQ16      1           
    X89       EQ50      -2          
    X89       EQ68      -1          
    X90       EQ19      -2          
    X90       EQ21      -1          
    X90       EQ26      -2          
    X90       EQ29      1           
    X90       EQ45      -2          
    X90       EQ52      -2          
    X91       EQ12      1           
    X91       EQ61      -1          
    X92       EQ38      1           
    X92       EQ72      1           
    X93       EQ6       -1          
    X93       EQ7       2           
    X93       EQ15      1           
    X93       EQ32      -1          
    X94       EQ11      1           
    X94       EQ16      1           
    X94       EQ35      -1          
    X94       EQ43      -2          
    X94       EQ51      2           
    X94       EQ58      2           
    X95       EQ5       -1          
    X95       EQ23      -1          
    X95       EQ43      2           
    X95       EQ46      -2          
    X95       EQ53      -1          
    X95       EQ69      2           
RHS
BOUNDS
 LO BOUND     X1        -1000       
 UP BOUND     X1        1000        
 LO BOUND     X2        -10         
 UP BOUND     X2        10          
 LO BOUND     X3        -1000       
 UP BOUND     X3        1000        
 LO BOUND     X4        -1000       
 UP BOUND     X4        1000        
 LO BOUND     X5        -1000       
 UP BOUND     X5        1000        
 LO BOUND     X6        -1000       
 UP BOUND     X6        1000        
 UP BOUND     X7        1000        
 LO BOUND     X8        -10         
 UP BOUND     X8        10          
 LO BOUND     X9        -1000       
 UP BOUND     X9        1000        
 UP BOUND     X10       1000        
 LO BOUND     X11       -10         
 UP BOUND     X11       10          
 LO BOUND     X12       -1000       
 UP BOUND     X12       1000        
 UP BOUND     X13       1000        
 LO BOUND     X14       -10         
 UP BOUND     X14       10          
 UP BOUND     X15       1000        
 LO BOUND     X16       -1000       
 UP BOUND     X16       1000        
 LO BOUND     X17       -1000       
 UP BOUND     X17       1000        
 LO BOUND     X18       -1000       
 UP BOUND     X18       1000        
 UP BOUND     X19       1000        
 LO BOUND     X20       -1000       
 UP BOUND     X20       1000        
 UP BOUND     X21       1000        
 LO BOUND     X22       -1000       
 UP BOUND     X22       1000        
 LO BOUND     X23       -1000       
 UP BOUND     X23       1000        
 LO BOUND     X24       -10         
 UP BOUND     X24       10          
 LO BOUND     X25       -1000       
 UP BOUND     X25       1000        
 LO BOUND     X26       -1000       
 UP BOUND     X26       1000        
 UP BOUND     X27       1000        
 LO BOUND     X28       -1000       
 UP BOUND     X28       1000        
 LO BOUND     X29       -1000       
 UP BOUND     X29       1000        
 UP BOUND     X30       1000        
 LO BOUND     X31       -10         
 UP BOUND     X31       10          
 UP BOUND     X32       1000        
 LO BOUND     X33       -1000       
 UP BOUND     X33       1000        
 LO BOUND     X34       -1000       
 UP BOUND     X34       1000        
 LO BOUND     X35       -1000       
 UP BOUND     X35       1000        
 LO BOUND     X36       -10         
 UP BOUND     X36       10          
 LO BOUND     X37       -10         
 UP BOUND     X37       10          
 UP BOUND     X38       1000        
 UP BOUND     X39       1000        
 LO BOUND     X40       -1000       
 UP BOUND     X40       1000        
 UP BOUND     X41       1000        
 LO BOUND     X42       -1000       
 UP BOUND     X42       1000        
 LO BOUND     X43       -1000       
 UP BOUND     X43       1000        
 UP BOUND     X44       1000        
 LO BOUND     X45       -1000       
 UP BOUND     X45       1000        
 LO BOUND     X46       -10         
 UP BOUND     X46       10          
 LO BOUND     X47       -1000       
 UP BOUND     X47       1000        
 LO BOUND     X48       -1000       
 UP BOUND     X48       1000        
 LO BOUND     X49       -10         
 UP BOUND     X49       10          
 LO BOUND     X50       -1000       
 UP BOUND     X50       1000        
 LO BOUND     X51       -1000       
 UP BOUND     X51       1000        
 LO BOUND     X52       -1000       
 UP BOUND     X52       1000        
 LO BOUND     X53       -10         
 UP BOUND     X53       10          
 LO BOUND     X54       -10         
 UP BOUND     X54       10          
 LO BOUND     X55       -1000       
 UP BOUND     X55       1000        
 LO BOUND     X56       -1000       
 UP BOUND     X56       1000        
 LO BOUND     X57       -1000       
 UP BOUND     X57       1000        
 LO BOUND     X58       -1000       
 UP BOUND     X58       1000        
 LO BOUND     X59       -1000       
 UP BOUND     X59       1000        
 UP BOUND     X60       1000        
 LO BOUND     X61       -1000       
 UP BOUND     X61       1000        
 LO BOUND     X62       -1000       
 UP BOUND     X62       1000        
 LO BOUND     X63       -1000       
 UP BOUND     X63       1000        
 LO BOUND     X64       -1000       
 UP BOUND     X64       1000        
 LO BOUND     X65       -1000       
 UP BOUND     X65       1000        
 LO BOUND     X66       -10         
 UP BOUND     X66       10          
 LO BOUND     X67       -1000       
 UP BOUND     X67       1000        
 LO BOUND     X68       -1000       
 UP BOUND     X68       1000        
 LO BOUND     X69       -1000       
 UP BOUND     X69       1000        
 UP BOUND     X70       1000        
 LO BOUND     X71       -1000       
 UP BOUND     X71       1000        
 LO BOUND     X72       -1000       
 UP BOUND     X72       1000        
 UP BOUND     X73       1000        
 LO BOUND     X74       -1000       
 UP BOUND     X74       1000        
 LO BOUND     X75       -1000       
 UP BOUND     X75       1000        
 LO BOUND     X76       -10         
 UP BOUND     X76       10          
 UP BOUND     X77       1000        
 LO BOUND     X78       -10         
 UP BOUND     X78       10          
 LO BOUND     X79       -10         
 UP BOUND     X79       10          
 LO BOUND     X80       -10         
 UP BOUND     X80       10          
 LO BOUND     X81       -1000       
 UP BOUND     X81       1000        
 LO BOUND     X82       -1000       
 UP BOUND     X82       1000        
 LO BOUND     X83       -1000       
 UP BOUND     X83       1000        
 LO BOUND     X84       -1000       
 UP BOUND     X84       1000        
 LO BOUND     X85       -1000       
 UP BOUND     X85       1000        
 LO BOUND     X86       -10         
 UP BOUND     X86       10          
 LO BOUND     X87       -1000       
 UP BOUND     X87       1000        
 LO BOUND     X88       -1000       
 UP BOUND     X88       1000        
 LO BOUND     X89       -10         
 UP BOUND     X89       10          
 UP BOUND     X90       1000        
 LO BOUND     X91       -10         
 UP BOUND     X91       10          
 UP BOUND     X92       1000        
 LO BOUND     X93       -1000       
 UP BOUND     X93       1000        
 LO BOUND     X94       -1000       
 UP BOUND     X94       1000        
 LO BOUND     X95       -1000       
 UP BOUND     X95       1000        
ENDATA
