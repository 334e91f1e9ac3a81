/*
 * Error-returning stand-ins for the twelve libuhd-backed radio entry points that
 * the reference link driver references (source/cpp_cuda/uhd_cpp/src/uhd_c_radio.h:18-99).
 *
 * TEST INFRASTRUCTURE ONLY.  This file exists so that the reference's CPU
 * receive path (uhd_ldpc_ofdm_link.cpp) links into the oracle harness without a
 * radio driver.  Nothing here is called on the paths the harness exposes; every
 * function reports "no radio" if it ever is.
 */
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "uhd_c_radio.h"

static int no_radio(char* err, size_t err_len)
{
    if (err != NULL && err_len > 0) {
        strncpy(err, "radio unavailable in the oracle harness", err_len - 1);
        err[err_len - 1] = '\0';
    }
    return -1;
}

int uhd_c_make_tx(uhd_c_radio_t** out, const char* args, double mclk, double rate, double freq,
                  double gain, const char* clk, const char* tsrc, const char* ant, const char* subdev,
                  const char* cpu_format, size_t channel, char* err, size_t err_len)
{
    (void)args; (void)mclk; (void)rate; (void)freq; (void)gain; (void)clk; (void)tsrc;
    (void)ant; (void)subdev; (void)cpu_format; (void)channel;
    if (out) *out = NULL;
    return no_radio(err, err_len);
}

int uhd_c_make_rx(uhd_c_radio_t** out, const char* args, double mclk, double rate, double freq,
                  double gain, const char* clk, const char* tsrc, const char* ant, const char* subdev,
                  size_t channel, char* err, size_t err_len)
{
    (void)args; (void)mclk; (void)rate; (void)freq; (void)gain; (void)clk; (void)tsrc;
    (void)ant; (void)subdev; (void)channel;
    if (out) *out = NULL;
    return no_radio(err, err_len);
}

int uhd_c_make_trx(uhd_c_radio_t** out, const char* args, double mclk, double rate, double freq,
                   double tx_gain, double rx_gain, const char* clk, const char* tsrc,
                   const char* tx_ant, const char* rx_ant, const char* tx_subdev, const char* rx_subdev,
                   const char* tx_cpu_format, size_t tx_channel, size_t rx_channel,
                   char* err, size_t err_len)
{
    (void)args; (void)mclk; (void)rate; (void)freq; (void)tx_gain; (void)rx_gain; (void)clk;
    (void)tsrc; (void)tx_ant; (void)rx_ant; (void)tx_subdev; (void)rx_subdev; (void)tx_cpu_format;
    (void)tx_channel; (void)rx_channel;
    if (out) *out = NULL;
    return no_radio(err, err_len);
}

void uhd_c_free(uhd_c_radio_t** radio)
{
    if (radio) *radio = NULL;
}

size_t uhd_c_tx_max_samps(uhd_c_radio_t* radio) { (void)radio; return 0; }
size_t uhd_c_rx_max_samps(uhd_c_radio_t* radio) { (void)radio; return 0; }

int uhd_c_tx_send(uhd_c_radio_t* radio, const void* samples, size_t nsamps, int start_of_burst,
                  int end_of_burst, double timeout, size_t* sent, char* err, size_t err_len)
{
    (void)radio; (void)samples; (void)nsamps; (void)start_of_burst; (void)end_of_burst; (void)timeout;
    if (sent) *sent = 0;
    return no_radio(err, err_len);
}

int uhd_c_rx_start(uhd_c_radio_t* radio, char* err, size_t err_len) { (void)radio; return no_radio(err, err_len); }
int uhd_c_rx_stop(uhd_c_radio_t* radio, char* err, size_t err_len) { (void)radio; return no_radio(err, err_len); }

int uhd_c_rx_recv(uhd_c_radio_t* radio, void* samples, size_t max_samps, double timeout,
                  size_t* received, int* status, char* err, size_t err_len)
{
    (void)radio; (void)samples; (void)max_samps; (void)timeout;
    if (received) *received = 0;
    if (status) *status = 3;
    return no_radio(err, err_len);
}

int uhd_c_pp_string(uhd_c_radio_t* radio, char* out, size_t out_len)
{
    (void)radio;
    if (out && out_len) out[0] = '\0';
    return -1;
}

int uhd_c_set_thread_priority(void) { return -1; }
