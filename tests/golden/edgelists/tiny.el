% a KONECT-style header
# a comment
1 2
2 1
2 3
3 3

 7 9
1	5
5 1
9 2
9 2
4 4
