/* Forced include for the reference build: glibc >= 2.30 declares gettid(),
 * which clashes with the reference's own static gettid (utils.h:105). */
#define _GNU_SOURCE
#include <unistd.h>
#define gettid ref_gettid
