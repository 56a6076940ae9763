// Emitted by Reffine's compile path (LoopGen, CanonPass, ReadWritePass, ScalarPass,
// CEmitter) for query `filter_sum` of oracle/ref/ref_queries.h, vectorize off; temporaries
// named after heap addresses renumbered.  Regenerate with oracle/ref/emit_generated.py.
// entry: filter_sum
#include <algorithm>
#include <cmath>
#include "reffine/vinstr/vinstr.h"

typedef struct {double _0; int64_t _1; } _0_t;

extern "C" void filter_sum(_0_t* output_addr, ArrowTable* lineitem) {
    int64_t _n0[int64_t(1)];
    int64_t* red_idx_addr_n1 = _n0;
    (red_idx_addr_n1)[int64_t(0)] = int64_t(0);
    red_idx_addr_n1;
    ;
    _0_t _n2[int64_t(1)];
    _0_t* state_addr_n3 = _n2;
    ((&state_addr_n3->_0))[int64_t(0)] = double(0.000000);
    (&state_addr_n3->_0);
    ((&state_addr_n3->_1))[int64_t(0)] = int64_t(0);
    (&state_addr_n3->_1);
    ;
    
    ;
    #pragma clang loop vectorize(enable) interleave(enable)
    while(1) {
        if (((red_idx_addr_n1)[int64_t(0)] >= get_array_len(get_array_child(get_vector_array(lineitem), uint32_t(1))))) break;
        
        if (get_null_bit((uint16_t*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(1)), uint32_t(0)), (red_idx_addr_n1)[int64_t(0)])) {
            ((&state_addr_n3->_0))[int64_t(0)] = ((((((((int32_t*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(730)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(1095))) && (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= double(0.050000))) && (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] <= double(0.070000))) && (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(4)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < double(24.000000))) ? (((&state_addr_n3->_0))[int64_t(0)] + (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(2)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] * ((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])) : ((&state_addr_n3->_0))[int64_t(0)]);
            (&state_addr_n3->_0);
            ((&state_addr_n3->_1))[int64_t(0)] = ((((((((int32_t*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(730)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(1095))) && (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= double(0.050000))) && (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] <= double(0.070000))) && (((double*) get_array_buf(get_array_child(get_vector_array(lineitem), uint32_t(4)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < double(24.000000))) ? (((&state_addr_n3->_1))[int64_t(0)] + int64_t(1)) : ((&state_addr_n3->_1))[int64_t(0)]);
            (&state_addr_n3->_1);
            ;
        } else {
        }
        ;
        (red_idx_addr_n1)[int64_t(0)] = ((red_idx_addr_n1)[int64_t(0)] + int64_t(1));
        red_idx_addr_n1;
        ;
        
    }
    
    _0_t* _red_loop_n4 = state_addr_n3;
    double red_0 = ((&_red_loop_n4->_0))[int64_t(0)];
    ((&output_addr->_0))[int64_t(0)] = red_0;
    (&output_addr->_0);
    int64_t red_1 = ((&_red_loop_n4->_1))[int64_t(0)];
    ((&output_addr->_1))[int64_t(0)] = red_1;
    (&output_addr->_1);
    ;
    ;
}