/* Second translation unit of the oldstyle program: old-style definitions and a global shared with
 * the first unit through the project header. */
#include <string.h>
#include "oldstyle.h"

int lib_calls = 0;

double scaled(v, factor)
    double v;
    int factor;
{
    lib_calls++;
    return v * factor;
}

int checksum(text)
    const char *text;
{
    int sum = 0, i;
    lib_calls++;
    for (i = 0; i < (int)strlen(text); i++)
        sum = sum * 31 + text[i];
    return sum;
}
