/* Declarations shared by oldstyle.c and oldstyle_lib.c (a project header: converted with them). */
#ifndef OLDSTYLE_H
#define OLDSTYLE_H

typedef struct record {
    int id;
    double value;
    char label[16];
} record;

extern int lib_calls;
double scaled(double v, int factor);
int checksum(const char* text);

#endif
