/* Declarations of the libconfig calls made by the EPREM reference's
 * configuration.c.  Defined by oracle/ref_shims.c, which reads the libconfig
 * file syntax; the per-operator harness never reads a file and fills the
 * reference's `config` struct directly.  Test infrastructure, not part of the
 * product. */
#ifndef EPREM_REFSHIM_LIBCONFIG_H
#define EPREM_REFSHIM_LIBCONFIG_H
typedef struct config_t { void *impl; } config_t;
typedef struct config_setting_t config_setting_t;
#define CONFIG_TRUE 1
#define CONFIG_FALSE 0
void config_init(config_t *);
void config_destroy(config_t *);
int config_read_file(config_t *, const char *);
int config_error_line(const config_t *);
const char *config_error_text(const config_t *);
int config_lookup_int(const config_t *, const char *, int *);
int config_lookup_float(const config_t *, const char *, double *);
int config_lookup_string(const config_t *, const char *, const char **);
config_setting_t *config_lookup(const config_t *, const char *);
double config_setting_get_float_elem(const config_setting_t *, int);
int config_setting_length(const config_setting_t *);
#endif
