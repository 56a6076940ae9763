// Emitted by Reffine's compile path (LoopGen, CanonPass, ReadWritePass, ScalarPass,
// CEmitter) for query `hashgroup_ree` of oracle/ref/ref_queries.h, vectorize off; temporaries
// named after heap addresses renumbered.  Regenerate with oracle/ref/emit_generated.py.
// entry: group_sum
#include <algorithm>
#include <cmath>
#include "reffine/vinstr/vinstr.h"

typedef struct {double _0; int64_t _1; } _0_t;

extern "C" void group_sum(ArrowTable** output_addr, ArrowTable* vec) {
    int64_t _n0[int64_t(1)];
    int64_t* _key_idx_addr = _n0;
    int64_t lb_n1 = ((int64_t*) get_array_buf(get_array_child(get_array_child(get_vector_array(vec), uint32_t(0)), uint32_t(1)), uint32_t(1)))[int64_t(0)];
    (_key_idx_addr)[int64_t(0)] = vector_locate(vec, lb_n1);
    _key_idx_addr;
    int64_t vec_len = get_array_len(get_array_child(get_array_child(get_vector_array(vec), uint32_t(0)), uint32_t(1)));
    vec_len;
    ;
    int64_t _n2[int64_t(1)];
    int64_t* _out_vec_idx_addr_n3 = _n2;
    (_out_vec_idx_addr_n3)[int64_t(0)] = int64_t(0);
    _out_vec_idx_addr_n3;
    int64_t _n4[int64_t(1)];
    int64_t* _null_count_n5 = _n4;
    (_null_count_n5)[int64_t(0)] = int64_t(0);
    _null_count_n5;
    ArrowTable* _out_vec_n6 = make_vector(int64_t(100000000), uint32_t(0));
    _out_vec_n6;
    bool _n7[int64_t(100000000)];
    bool* _bytemap_n8 = _n7;
    _bytemap_n8;
    
    ;
    #pragma clang loop vectorize(enable) interleave(enable)
    while(1) {
        if (!((_key_idx_addr)[int64_t(0)] < vec_len)) break;
        
        bool valid_n9 = get_null_bit((uint16_t*) get_array_buf(get_array_child(get_array_child(get_vector_array(vec), uint32_t(0)), uint32_t(1)), uint32_t(0)), (_key_idx_addr)[int64_t(0)]);
        bool _body_cond_n10 = (((_key_idx_addr)[int64_t(0)] < vec_len) && valid_n9);
        if (_body_cond_n10) {
            int64_t _key = ((int64_t*) get_array_buf(get_array_child(get_array_child(get_vector_array(vec), uint32_t(0)), uint32_t(1)), uint32_t(1)))[(_key_idx_addr)[int64_t(0)]];
            int64_t key = _key;
            ((int64_t*) get_array_buf(get_array_child(get_vector_array(_out_vec_n6), uint32_t(0)), uint32_t(1)))[(_out_vec_idx_addr_n3)[int64_t(0)]] = key;
            (int64_t*) get_array_buf(get_array_child(get_vector_array(_out_vec_n6), uint32_t(0)), uint32_t(1));
            int64_t _n11[int64_t(1)];
            int64_t* red_idx_addr_n12 = _n11;
            (red_idx_addr_n12)[int64_t(0)] = read_runend_buf((int32_t*) get_array_buf(get_array_child(get_array_child(get_vector_array(vec), uint32_t(0)), uint32_t(0)), uint32_t(1)), ((_key_idx_addr)[int64_t(0)] - int64_t(1)));
            red_idx_addr_n12;
            ;
            _0_t _n13[int64_t(1)];
            _0_t* state_addr_n14 = _n13;
            ((&state_addr_n14->_0))[int64_t(0)] = double(0.000000);
            (&state_addr_n14->_0);
            ((&state_addr_n14->_1))[int64_t(0)] = int64_t(0);
            (&state_addr_n14->_1);
            ;
            
            ;
            #pragma clang loop vectorize(enable) interleave(enable)
            while(1) {
                if (((red_idx_addr_n12)[int64_t(0)] >= read_runend_buf((int32_t*) get_array_buf(get_array_child(get_array_child(get_vector_array(vec), uint32_t(0)), uint32_t(0)), uint32_t(1)), (_key_idx_addr)[int64_t(0)]))) break;
                
                if (get_null_bit((uint16_t*) get_array_buf(get_array_child(get_vector_array(vec), uint32_t(1)), uint32_t(0)), (red_idx_addr_n12)[int64_t(0)])) {
                    ((&state_addr_n14->_0))[int64_t(0)] = (((&state_addr_n14->_0))[int64_t(0)] + ((double*) get_array_buf(get_array_child(get_vector_array(vec), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n12)[int64_t(0)]]);
                    (&state_addr_n14->_0);
                    ((&state_addr_n14->_1))[int64_t(0)] = (((&state_addr_n14->_1))[int64_t(0)] + int64_t(1));
                    (&state_addr_n14->_1);
                    ;
                } else {
                }
                ;
                (red_idx_addr_n12)[int64_t(0)] = ((red_idx_addr_n12)[int64_t(0)] + int64_t(1));
                red_idx_addr_n12;
                ;
                
            }
            
            _0_t* _red_loop_n15 = state_addr_n14;
            double agg_0 = ((&_red_loop_n15->_0))[int64_t(0)];
            ((double*) get_array_buf(get_array_child(get_vector_array(_out_vec_n6), uint32_t(1)), uint32_t(1)))[(_out_vec_idx_addr_n3)[int64_t(0)]] = agg_0;
            (double*) get_array_buf(get_array_child(get_vector_array(_out_vec_n6), uint32_t(1)), uint32_t(1));
            int64_t agg_1 = ((&_red_loop_n15->_1))[int64_t(0)];
            ((int64_t*) get_array_buf(get_array_child(get_vector_array(_out_vec_n6), uint32_t(2)), uint32_t(1)))[(_out_vec_idx_addr_n3)[int64_t(0)]] = agg_1;
            (int64_t*) get_array_buf(get_array_child(get_vector_array(_out_vec_n6), uint32_t(2)), uint32_t(1));
            ;
            (_out_vec_idx_addr_n3)[int64_t(0)] = ((_out_vec_idx_addr_n3)[int64_t(0)] + int64_t(1));
            _out_vec_idx_addr_n3;
        } else {
        }
        ;
        (_key_idx_addr)[int64_t(0)] = ((_key_idx_addr)[int64_t(0)] + int64_t(1));
        _key_idx_addr;
        ;
        
    }
    finalize_vector(_out_vec_n6, _bytemap_n8, (_out_vec_idx_addr_n3)[int64_t(0)], (_null_count_n5)[int64_t(0)])
    ;
    
    ArrowTable* _loop_n16 = _out_vec_n6;
    ArrowTable* op = _loop_n16;
    (output_addr)[int64_t(0)] = op;
    output_addr;
    ;
}